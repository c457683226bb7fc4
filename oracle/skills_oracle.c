/*
 * skills_oracle.c -- CPU ORACLE (test infrastructure only).
 *
 * Plain-C restatement of the Ski-LLS solve path used as the parity checker
 * for the GPU solver.  Only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / reference arm may load this library; the product path never
 * calls it.  Every function names the reference file:line it restates.
 *
 * Parity pins (see tests/test_oracle_*.py):
 *   - the random stream is checked against the host C library's rand()
 *     (glibc TYPE_3 additive generator, the RNG the reference calls);
 *   - gen_hashing_matrix is checked against the reference's own translation
 *     unit (src/sparse_helpers.cpp) when oracle/_ref has been built;
 *   - the full solvers are checked against the known answers of
 *     test/ski-llsDenseExample.cpp:48, test/ski-llsSparseExample.cpp:58 and
 *     the expected residuals of test/test_solvers.sh:138-139.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

/* ------------------------------------------------------------------------ */
/* glibc-compatible rand(): TYPE_3 additive feedback generator, degree 31,  */
/* separation 3.  Restated from the published description of glibc's        */
/* random_r.c (srandom_r seeding with the 16807 Lehmer LCG via Schrage's     */
/* method, 310 discarded outputs, output = state word >> 1).  The reference */
/* draws hash rows and signs from it: src/sparse_helpers.cpp:74-115,        */
/* src/dense_helpers.cpp:7-16.                                              */
/* ------------------------------------------------------------------------ */
typedef struct {
    int32_t s[31];
    int32_t f, r;           /* front / rear cursor into s[] */
} orc_rng;

void orc_rng_seed(orc_rng* g, uint32_t seed)
{
    if (seed == 0) seed = 1;
    int32_t word = (int32_t)seed;
    g->s[0] = word;
    for (int i = 1; i < 31; ++i) {
        /* 16807 * word mod (2^31-1) without overflow (Schrage). */
        long hi = word / 127773;
        long lo = word % 127773;
        long w = 16807 * lo - 2836 * hi;
        if (w < 0) w += 2147483647;
        word = (int32_t)w;
        g->s[i] = word;
    }
    g->f = 3;
    g->r = 0;
    for (int i = 0; i < 310; ++i) {
        uint32_t v = (uint32_t)g->s[g->f] + (uint32_t)g->s[g->r];
        g->s[g->f] = (int32_t)v;
        g->f = (g->f + 1) % 31;
        g->r = (g->r + 1) % 31;
    }
}

int32_t orc_rng_next(orc_rng* g)
{
    uint32_t v = (uint32_t)g->s[g->f] + (uint32_t)g->s[g->r];
    g->s[g->f] = (int32_t)v;
    g->f = (g->f + 1) % 31;
    g->r = (g->r + 1) % 31;
    return (int32_t)(v >> 1);
}

size_t orc_rng_size(void) { return sizeof(orc_rng); }

void orc_rng_fill(orc_rng* g, int64_t count, int32_t* out)
{
    for (int64_t i = 0; i < count; ++i) out[i] = orc_rng_next(g);
}

/* ------------------------------------------------------------------------ */
/* gen_hashing_matrix + select_k_from_n + gen_0_to_n                        */
/* (src/sparse_helpers.cpp:66-116).  S is m x n with k entries per column.   */
/* Column i takes k distinct rows by a partial Fisher-Yates shuffle of a     */
/* permutation array that persists across columns; all n*k signs are drawn   */
/* after all row indices.  rows[i*k+j], vals[i*k+j] = +-1/sqrt(k).           */
/* ------------------------------------------------------------------------ */
int orc_gen_hashing(orc_rng* g, int64_t m, int64_t n, int64_t k,
                    int64_t* rows, double* vals)
{
    if (k > m || k < 1) return -1;
    int64_t* perm = (int64_t*)malloc((size_t)m * sizeof(int64_t));
    if (!perm) return -2;
    for (int64_t i = 0; i < m; ++i) perm[i] = i;
    for (int64_t i = 0; i < n; ++i) {
        for (int64_t j = 0; j < k; ++j) {
            int64_t t = (int64_t)orc_rng_next(g) % (m - j) + j;
            int64_t tmp = perm[t];
            perm[t] = perm[j];
            perm[j] = tmp;
        }
        for (int64_t j = 0; j < k; ++j) rows[i * k + j] = perm[j];
    }
    double inv = 1.0 / sqrt((double)k);
    for (int64_t i = 0; i < n * k; ++i)
        vals[i] = inv * (double)((orc_rng_next(g) % 2) * 2 - 1);
    free(perm);
    return 0;
}

/* Random +-1 signs, src/dense_helpers.cpp:7-16 (scale = 1). */
void orc_rand_signs(orc_rng* g, int64_t n, double scale, double* out)
{
    for (int64_t i = 0; i < n; ++i)
        out[i] = scale * (double)((orc_rng_next(g) % 2) * 2 - 1);
}

/* ------------------------------------------------------------------------ */
/* Sparse sketch SA = S*A (dense m x d column-major output) and S*b.        */
/* Restates sparse_sketch (src/sketching.cpp:90-112): cs_dl_multiply visits */
/* A column by column, each nonzero A(i,j) scattering into the k hashed rows */
/* of S's column i in stored order; cs_dl_gaxpy accumulates b the same way.  */
/* ------------------------------------------------------------------------ */
void orc_sparse_sketch(int64_t n, int64_t d, const int64_t* Ap, const int64_t* Ai,
                       const double* Ax, const double* b,
                       int64_t m, int64_t k, const int64_t* hrows, const double* hvals,
                       double* SA /* m*d, col-major */, double* Sb /* m */)
{
    (void)n;
    memset(SA, 0, (size_t)(m * d) * sizeof(double));
    for (int64_t j = 0; j < d; ++j) {
        double* col = SA + j * m;
        for (int64_t p = Ap[j]; p < Ap[j + 1]; ++p) {
            int64_t i = Ai[p];
            double a = Ax[p];
            for (int64_t t = 0; t < k; ++t)
                col[hrows[i * k + t]] += hvals[i * k + t] * a;
        }
    }
    if (b && Sb) {
        memset(Sb, 0, (size_t)m * sizeof(double));
        for (int64_t i = 0; i < n; ++i)
            for (int64_t t = 0; t < k; ++t)
                Sb[hrows[i * k + t]] += hvals[i * k + t] * b[i];
    }
}

/* Dense sketch SA = alpha*S*Y, alpha = 1/sqrt(k) on top of S's +-1/sqrt(k)  */
/* values (src/sketching.cpp:39-62 -> SpMat_Op::mm -> csc_mv 'n',           */
/* src/SpMat.cpp:37-56): y[row] += (alpha*a)*x[i] in column order of S.     */
void orc_dense_sketch(int64_t N, int64_t d, const double* Y, int64_t ldy,
                      int64_t m, int64_t k, const int64_t* hrows, const double* hvals,
                      double* SA /* m*d */)
{
    double alpha = 1.0 / sqrt((double)k);
    memset(SA, 0, (size_t)(m * d) * sizeof(double));
    for (int64_t j = 0; j < d; ++j) {
        const double* y = Y + j * ldy;
        double* col = SA + j * m;
        for (int64_t i = 0; i < N; ++i)
            for (int64_t t = 0; t < k; ++t)
                col[hrows[i * k + t]] += alpha * hvals[i * k + t] * y[i];
    }
}

/* ------------------------------------------------------------------------ */
/* Triangular solves with the upper-triangular R (r x r, column-major, ld). */
/* Column-oriented back substitution in the order of                        */
/* cs_usolve_cholmod_structure / cs_utsolve_cholmod_structure               */
/* (src/sparse_helpers.cpp:122-181); perturb is added to each pivot when     */
/* success == 0.  The dense path's dtrsv (src/IterSolver.cpp:89,95) is the   */
/* same arithmetic with perturb = 0.                                         */
/* ------------------------------------------------------------------------ */
void orc_usolve(int64_t r, const double* R, int64_t ld, double* x, int success, double perturb)
{
    for (int64_t j = r - 1; j >= 0; --j) {
        double piv = R[j + j * ld];
        if (!success) piv += perturb;
        x[j] /= piv;
        const double* col = R + j * ld;
        double xj = x[j];
        for (int64_t i = 0; i < j; ++i) x[i] -= col[i] * xj;
    }
}

void orc_utsolve(int64_t r, const double* R, int64_t ld, double* x, int success, double perturb)
{
    for (int64_t j = 0; j < r; ++j) {
        const double* col = R + j * ld;
        double s = x[j];
        for (int64_t i = 0; i < j; ++i) s -= col[i] * x[i];
        double piv = R[j + j * ld];
        if (!success) piv += perturb;
        x[j] = s / piv;
    }
}

/* CSC mat-vec, src/SpMat.cpp:37-74 (beta handled by the caller). */
static void csc_mv_n(int64_t nrow, int64_t ncol, const int64_t* Ap, const int64_t* Ai,
                     const double* Ax, double alpha, const double* x, double beta, double* y)
{
    if (beta == 0.0) memset(y, 0, (size_t)nrow * sizeof(double));
    else for (int64_t i = 0; i < nrow; ++i) y[i] *= beta;
    for (int64_t j = 0; j < ncol; ++j)
        for (int64_t p = Ap[j]; p < Ap[j + 1]; ++p) y[Ai[p]] += alpha * Ax[p] * x[j];
}

static void csc_mv_t(int64_t nrow, int64_t ncol, const int64_t* Ap, const int64_t* Ai,
                     const double* Ax, double alpha, const double* x, double beta, double* y)
{
    (void)nrow;
    if (beta == 0.0) memset(y, 0, (size_t)ncol * sizeof(double));
    else for (int64_t j = 0; j < ncol; ++j) y[j] *= beta;
    for (int64_t j = 0; j < ncol; ++j)
        for (int64_t p = Ap[j]; p < Ap[j + 1]; ++p) y[j] += alpha * Ax[p] * x[Ai[p]];
}

void orc_csc_mv(char trans, int64_t nrow, int64_t ncol, const int64_t* Ap, const int64_t* Ai,
                const double* Ax, double alpha, const double* x, double beta, double* y)
{
    if (trans == 'n') csc_mv_n(nrow, ncol, Ap, Ai, Ax, alpha, x, beta, y);
    else csc_mv_t(nrow, ncol, Ap, Ai, Ax, alpha, x, beta, y);
}

/* dense column-major gemv y = alpha*op(A)*x + beta*y (dgemv semantics). */
static void dense_mv(char trans, int64_t nrow, int64_t ncol, const double* A, int64_t lda,
                     double alpha, const double* x, double beta, double* y)
{
    if (trans == 'n') {
        if (beta == 0.0) memset(y, 0, (size_t)nrow * sizeof(double));
        else for (int64_t i = 0; i < nrow; ++i) y[i] *= beta;
        for (int64_t j = 0; j < ncol; ++j) {
            double t = alpha * x[j];
            const double* a = A + j * lda;
            for (int64_t i = 0; i < nrow; ++i) y[i] += t * a[i];
        }
    } else {
        for (int64_t j = 0; j < ncol; ++j) {
            const double* a = A + j * lda;
            double s = 0.0;
            for (int64_t i = 0; i < nrow; ++i) s += a[i] * x[i];
            y[j] = (beta == 0.0 ? 0.0 : beta * y[j]) + alpha * s;
        }
    }
}

static double nrm2(int64_t n, const double* x)
{
    /* scaled sum of squares (dnrm2 semantics, no overflow for finite data) */
    double scale = 0.0, ssq = 1.0;
    for (int64_t i = 0; i < n; ++i) {
        if (x[i] != 0.0) {
            double a = fabs(x[i]);
            if (scale < a) { ssq = 1.0 + ssq * (scale / a) * (scale / a); scale = a; }
            else ssq += (a / scale) * (a / scale);
        }
    }
    return scale * sqrt(ssq);
}

/* ------------------------------------------------------------------------ */
/* Preconditioned LSQR, src/IterSolver.cpp:160-284 with the operator         */
/* Abar = A(:,cols) * R^{-1} of LinOP_sparse_preconditioner (:21-63) or      */
/* LinOP_dense_preconditioner (:66-108).  A is either CSC (Ap != NULL) or    */
/* dense column-major (Ad).  cols (length r) selects and orders the columns  */
/* of A (the pivoted subset A*P1); R is r x r upper triangular (ld ldr).     */
/* Outputs y (length r), flag (0 converged, 1 max_it), it.                   */
/* ------------------------------------------------------------------------ */
typedef struct {
    int64_t n, d;
    const int64_t *Ap, *Ai; const double* Ax;     /* CSC, or */
    const double* Ad; int64_t lda;                 /* dense   */
    const int64_t* cols; int64_t r;
    const double* R; int64_t ldr;
    int success; double perturb;
    double* tmp_r;  /* r */
    double* tmp_d;  /* d */
} orc_op;

/* y = alpha * A(:,cols) * R^{-1} x + beta * y */
static void op_n(orc_op* o, double alpha, const double* x, double beta, double* y)
{
    memcpy(o->tmp_r, x, (size_t)o->r * sizeof(double));
    orc_usolve(o->r, o->R, o->ldr, o->tmp_r, o->success, o->perturb);
    if (o->Ap) {
        /* Areduced = A(:, cols) as a CSC with the selected columns */
        if (beta == 0.0) memset(y, 0, (size_t)o->n * sizeof(double));
        else for (int64_t i = 0; i < o->n; ++i) y[i] *= beta;
        for (int64_t c = 0; c < o->r; ++c) {
            int64_t j = o->cols[c];
            for (int64_t p = o->Ap[j]; p < o->Ap[j + 1]; ++p)
                y[o->Ai[p]] += alpha * o->Ax[p] * o->tmp_r[c];
        }
    } else {
        if (beta == 0.0) memset(y, 0, (size_t)o->n * sizeof(double));
        else for (int64_t i = 0; i < o->n; ++i) y[i] *= beta;
        for (int64_t c = 0; c < o->r; ++c) {
            const double* a = o->Ad + o->cols[c] * o->lda;
            double t = alpha * o->tmp_r[c];
            for (int64_t i = 0; i < o->n; ++i) y[i] += t * a[i];
        }
    }
}

/* y = alpha * R^{-T} A(:,cols)^T x + beta * y */
static void op_t(orc_op* o, double alpha, const double* x, double beta, double* y)
{
    for (int64_t c = 0; c < o->r; ++c) {
        int64_t j = o->cols[c];
        double s = 0.0;
        if (o->Ap) {
            for (int64_t p = o->Ap[j]; p < o->Ap[j + 1]; ++p) s += 1.0 * o->Ax[p] * x[o->Ai[p]];
        } else {
            const double* a = o->Ad + j * o->lda;
            for (int64_t i = 0; i < o->n; ++i) s += a[i] * x[i];
        }
        o->tmp_r[c] = s;
    }
    orc_utsolve(o->r, o->R, o->ldr, o->tmp_r, o->success, o->perturb);
    for (int64_t c = 0; c < o->r; ++c) y[c] = beta * y[c] + alpha * o->tmp_r[c];
}

int orc_lsqr(int64_t n, int64_t d,
             const int64_t* Ap, const int64_t* Ai, const double* Ax,
             const double* Ad, int64_t lda,
             const int64_t* cols, int64_t r, const double* R, int64_t ldr,
             int success, double perturb,
             const double* b, double tol, int64_t max_it,
             double* x /* r */, int* flag, int64_t* it)
{
    orc_op o = {n, d, Ap, Ai, Ax, Ad, lda, cols, r, R, ldr, success, perturb, NULL, NULL};
    double* buf = (double*)malloc((size_t)(n + 4 * r + 1) * sizeof(double));
    if (!buf) return -2;
    double* u = buf;
    double* v = u + n;
    double* w = v + r;
    o.tmp_r = w + r;
    memset(v, 0, (size_t)r * sizeof(double));
    memset(w, 0, (size_t)r * sizeof(double));
    memcpy(u, b, (size_t)n * sizeof(double));
    double alpha = 0.0;
    double beta = nrm2(n, u);
    if (beta > 0) {
        for (int64_t i = 0; i < n; ++i) u[i] *= 1.0 / beta;
        op_t(&o, 1.0, u, 0.0, v);
        alpha = nrm2(r, v);
    }
    if (alpha > 0) {
        for (int64_t i = 0; i < r; ++i) v[i] *= 1.0 / alpha;
        memcpy(w, v, (size_t)r * sizeof(double));
    }
    memset(x, 0, (size_t)r * sizeof(double));
    double nrm_ar = alpha * beta;
    if (nrm_ar == 0) { *it = 0; *flag = 0; free(buf); return 0; }
    double phibar = beta, rhobar = alpha, nrm_a = 0.0;
    *flag = 1; *it = 0;
    for (int64_t kk = 0; kk < max_it; ++kk) {
        (*it)++;
        op_n(&o, 1.0, v, -alpha, u);
        beta = nrm2(n, u);
        if (beta > 0) {
            for (int64_t i = 0; i < n; ++i) u[i] *= 1.0 / beta;
            nrm_a = sqrt(nrm_a * nrm_a + alpha * alpha + beta * beta);
            op_t(&o, 1.0, u, -beta, v);
            alpha = nrm2(r, v);
            if (alpha > 0) for (int64_t i = 0; i < r; ++i) v[i] *= 1.0 / alpha;
        }
        double rho = sqrt(rhobar * rhobar + beta * beta);
        double cs = rhobar / rho, sn = beta / rho;
        double theta = sn * alpha;
        rhobar = -cs * alpha;
        double phi = cs * phibar;
        phibar = sn * phibar;
        double t1 = phi / rho, t2 = -theta / rho;
        for (int64_t i = 0; i < r; ++i) x[i] += t1 * w[i];
        for (int64_t i = 0; i < r; ++i) w[i] = t2 * w[i] + v[i];
        double nrm_r = phibar;
        nrm_ar = phibar * alpha * fabs(cs);
        if (nrm_ar < tol * nrm_a * nrm_r) { *flag = 0; break; }
    }
    free(buf);
    return 0;
}

/* Residual helpers used by the solver restatements and tests. */
void orc_csc_residual(int64_t n, int64_t d, const int64_t* Ap, const int64_t* Ai, const double* Ax,
                      const double* x, const double* b, double* r)
{
    memcpy(r, b, (size_t)n * sizeof(double));
    csc_mv_n(n, d, Ap, Ai, Ax, -1.0, x, 1.0, r);
}

void orc_dense_residual(int64_t n, int64_t d, const double* A, int64_t lda,
                        const double* x, const double* b, double* r)
{
    memcpy(r, b, (size_t)n * sizeof(double));
    dense_mv('n', n, d, A, lda, -1.0, x, 1.0, r);
}
