/*
 * skills_gb300.h -- C ABI of the GB300 (sm_103a) Ski-LLS solver.
 *
 * Plain pointers and sizes only; no exceptions cross this boundary.  Every
 * entry point returns an skl_status and, on failure, leaves a message for
 * skl_last_error().  The C++ drop-in header ski-lls.h re-exposes the three
 * reference signatures over these calls.
 *
 * Reference interfaces replaced (file:line in numericalalgorithmsgroup/Ski-LLS):
 *   skl_sparse_solve  <- ls_sparse_spqr                 include/ski-lls.h:24-28,
 *                                                        src/ls_sparse_spqr.cpp:79-214
 *   skl_dense_solve   <- ls_dense_hashing_blendenpik    include/ski-lls.h:15-17,
 *                                                        src/ls_dense_hashing_blendenpik.cpp:23-149
 *   skl_dense_solve with opts.use_cpqr = 0
 *                     <- ls_dense_hashing_blendenpik_noCPQR  include/ski-lls.h:19-21
 *   skl_dense_blendenpik_solve
 *                     <- ls_dense_blendenpik            include/blendenpik.hpp:31-33,
 *                                                        src/ls_dense_blendenpik.cpp:21-70
 *   skl_subsample_rows <- random_sample's row draw      src/dense_helpers.cpp:19-39
 *   skl_srand / skl_hash_generate
 *                     <- srand() + gen_hashing_matrix   src/sparse_helpers.cpp:66-116
 *   skl_sketch_sparse <- sparse_sketch(A,k,gamma,b,bs)  src/sketching.cpp:90-112
 *   skl_sketch_dense  <- rand_hashing_dct(A,b,..)       src/dense_helpers.cpp:83-112
 *   skl_dht           <- fast_unitary_transform         src/fast_unitary_transform.cpp:42-121
 *   skl_cpqr          <- column_pivoted_qr(A,E,tau)     src/column_pivoted_QR.cpp:35-58
 *   skl_trsv_upper    <- cs_usolve/utsolve_cholmod_structure, dtrsv
 *                                                        src/sparse_helpers.cpp:122-181,
 *                                                        src/IterSolver.cpp:89,95
 *   skl_csc_mv        <- csc_mv 'n' / 't' (CSC_Mat::mv)  src/SpMat.cpp:37-74,
 *                                                        include/SpMat.hpp:132-136
 *   skl_gemm_vta      <- the W = C^T V product of dlarfb in NoFLA_Apply_Q_WY_lhfc_blk_var4
 *                        hqrrp/lapack_compatible_sources/NoFLA_HQRRP_WY_blk_var4_skint.c:721-746
 *   skl_gemm_update   <- the C -= V W^T product of the same dlarfb call
 */
#ifndef SKILLS_GB300_H
#define SKILLS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    SKL_OK = 0,
    SKL_ERR_INVALID = 1,            /* bad argument (null pointer, size, csc structure) */
    SKL_ERR_NOT_OVERDETERMINED = 2, /* rows < cols: "Matrix is not overdetermined." */
    SKL_ERR_RANK_ZERO = 3,          /* factorization found rank 0: "SPQR Factorization fails" */
    SKL_ERR_CUDA = 4,               /* CUDA runtime error */
    SKL_ERR_NO_DEVICE = 5,          /* no usable sm_103 device */
    SKL_ERR_TIMEOUT = 6,            /* a bounded device-side wait gave up */
    SKL_ERR_ALLOC = 7,              /* device or host allocation failed */
    SKL_ERR_NONFINITE = 8           /* NaN/Inf in A or b */
} skl_status;

typedef enum { SKL_PREC_MIXED = 0, SKL_PREC_FP64 = 1 } skl_precision;

/* Compressed sparse column matrix with the cs_dl field layout of CSparse
 * (m rows, n cols, p[n+1] column pointers, i[nnz] row indices, x[nnz]
 * values, 64-bit integers), as the reference passes it
 * (test/ski-llsSparseExample.cpp:15-20). */
typedef struct {
    int64_t m, n, nzmax;
    const int64_t* p;
    const int64_t* i;
    const double* x;
} skl_csc;

typedef struct {
    double gamma;            /* over-sampling ratio, m = ceil(gamma*d)           */
    int64_t k;               /* nonzeros per column of the hashing matrix        */
    double abs_tol;          /* early exit if ||b - A xs|| < abs_tol             */
    double it_tol;           /* LSQR relative tolerance                           */
    int64_t max_it;          /* LSQR iteration limit                              */
    double rcond_threshold;  /* sparse path: preconditioner 'well conditioned'    */
    double perturb;          /* sparse path: pivot perturbation when ill cond.    */
    double rcond;            /* dense path: minimal |R_ii| kept (absolute rule)   */
    double rank_tol;         /* sparse path: relative rank tolerance on |R_ii|;
                                <= 0 selects 20*(m+d)*eps_64 (SPQR's default) on
                                the FP64 path and 2*sqrt(m)*eps_32 on the mixed
                                path, which keeps the columns below it in LSQR's
                                basis (skl_info.unresolved_cols); > 0 drops them */
    int precision;           /* skl_precision                                     */
    int use_cpqr;            /* dense path: 1 = CPQR + rank (ls_dense_hashing_blendenpik),
                                0 = unpivoted QR (..._noCPQR)                     */
    int seed_mode;           /* 0: continue the library's glibc-compatible stream
                                   (sparse path; a fresh process is seed 1),
                                1: reseed with `seed` before drawing              */
    uint32_t seed;           /* dense path seed (the reference uses time(NULL));
                                0 selects time(NULL)                              */
    int wisdom;              /* dense path: pad the DHT length to a 2^a3^b5^c size */
    double backward_tol;     /* >0: keep iterating until ||A^T r||/(||A||_F||r||)
                                <= backward_tol (checked in FP64)                 */
    int64_t max_refine;      /* restarts allowed to meet backward_tol            */
    int device;              /* CUDA device ordinal                               */
    void* stream;            /* cudaStream_t to run on; NULL = the library's own  */
    int profile;             /* 1: time the LSQR products with CUDA events        */
    int autotune;            /* sparse path, 1: the first solve of a shape class
                                times the candidate launch shapes (sketch block
                                size, CPQR panel width, lanes per row / column of
                                the two sparse products) on its own data and caches
                                the fastest for the process; 0: fixed heuristics */
} skl_opts;

typedef struct {
    int64_t rank;            /* detected rank                                     */
    int flag;                /* 0 = converged or early exit, 1 = max_it reached   */
    int64_t it;              /* LSQR iterations (0 on early exit)                 */
    int success;             /* sparse path: rcond(R11) > rcond_threshold         */
    int64_t sketch_rows;     /* m                                                 */
    double rcond_r11;        /* 1/(||R11||_inf ||R11^{-1}||_inf)                   */
    double explicit_residual;/* ||b - A xs|| of the sketch solution               */
    double residual_norm;    /* ||b - A x|| (FP64)                                */
    double backward_error;   /* ||A^T r|| / (||A||_F ||r||) (FP64)                */
    double t_total_ms;       /* device time of the whole solve (CUDA events)      */
    double t_upload_ms;      /* host->device copies                               */
    double t_setup_ms;       /* format conversion, norms, hashing upload          */
    double t_sketch_ms;      /* S*A, S*b (and DHT on the dense path)              */
    double t_qr_ms;          /* randomized CPQR + Q^T c                           */
    double t_precond_ms;     /* rank, R11^{-1}, condition estimate, explicit x    */
    double t_lsqr_ms;        /* LSQR iterations                                   */
    double t_host_hash_ms;   /* host wall time generating the hash stream         */
    int64_t kernel_launches; /* kernels launched by this solve                    */
    /* opts.profile = 1: summed CUDA-event time and launch count of the LSQR
       products (0: A*z CSR/dense, 1: A^T*u CSC/dense, 2: M*v, 3: M^T*t) */
    double prof_ms[4];
    int64_t prof_launches[4];
    /* opts.profile = 1: CUDA-event ms of the QR sub-steps: 0 sample QRP,
       1 column moves, 2 panel, 3 Q^T c, 4 W = V^T A, 5 Z = T^T W,
       6 A -= V Z, 7 sample downdate, 8 initial sample Y = G A */
    double qr_prof_ms[9];
    /* mixed path: refinement steps of the explicit sketch solution against
       the FP64 residual (each ||b - A xs|| at least halved) */
    int64_t sketch_refine_steps;
    /* mixed sparse path: pivoted columns whose |R_ii| lies below what the
       FP32 factorization resolves (2 sqrt(m) eps_32 |R_00|).  They are not
       dropped: LSQR carries them with unit preconditioning, so its FP64-class
       iteration decides whether they reduce the residual.  Not counted in
       `rank`. */
    int64_t unresolved_cols;
    /* mixed dense path: 1 if A held values outside [2^-100, 2^100] in
       magnitude and the solve ran on the FP64 path instead */
    int fp64_fallback;
    /* launch shapes this solve used: sketch block size, CPQR panel width,
       lanes per CSR row of A z, lanes per CSC column of A^T u.  The panel width
       is always reported on the mixed path (0 on the FP64 path); the others
       are 0 unless autotuned (0 = the fixed heuristic) */
    int64_t tuned[4];
} skl_info;

/* Defaults of include/bench_config.hpp:7-20 (IT_TOL 1e-6, MAX_IT 10000,
 * gamma 1.1, k 3, PERTURB 1e-10, RCOND_THRESHOLD 1e-10, ABS_TOL 1e-8). */
void skl_default_opts(skl_opts* opts);

/* Message of the last failing call on this thread ("" if none). */
const char* skl_last_error(void);

/* Library version string. */
const char* skl_version(void);

/* Reseed the library's glibc-compatible random stream (srand semantics). */
void skl_srand(uint32_t seed);

/* ---------------------------------------------------------------- solvers */

/* Sparse least squares min ||Ax-b||, A in CSC (host memory).  x (host, A->n
 * entries) receives the solution.  Sketch: s-hashing with opts->k nonzeros
 * per column, m = ceil(gamma*n); CPQR of the sketch; LSQR preconditioned by
 * R11. */
skl_status skl_sparse_solve(const skl_csc* A, const double* b, double* x,
                            const skl_opts* opts, skl_info* info);

/* Same with A, b and x already in device memory (CSC with 64-bit indices). */
skl_status skl_sparse_solve_device(const skl_csc* A_dev, const double* b_dev, double* x_dev,
                                   const skl_opts* opts, skl_info* info);

/* Dense least squares, A column-major n x d with leading dimension lda (host). */
skl_status skl_dense_solve(const double* A, int64_t lda, int64_t n, int64_t d,
                           const double* b, double* x, const skl_opts* opts, skl_info* info);

/* nprob independent sparse problems (host buffers, each as for
 * skl_sparse_solve) with one set of options.  No counterpart in the reference
 * (it solves one problem per call); it serves batched workloads of many small
 * problems, which a single solve cannot keep the GPU busy with.  The hashing
 * of every problem is drawn in problem order exactly as a loop of
 * skl_sparse_solve calls with the same options would draw it, so each x[p] is
 * bit-identical to that loop's; the problems then run concurrently on worker
 * threads, each with its own stream (SKILLS_BATCH_STREAMS, default 8;
 * opts->stream is not used).  info[p] and status[p] (both optional) per
 * problem; the return value is the first failing problem's status. */
skl_status skl_batched_sparse_solve(int64_t nprob, const skl_csc* A, const double* const* b,
                                    double* const* x, const skl_opts* opts, skl_info* info,
                                    skl_status* status);

/* Same with A, b, x in device memory. */
skl_status skl_dense_solve_device(const double* A_dev, int64_t lda, int64_t n, int64_t d,
                                  const double* b_dev, double* x_dev, const skl_opts* opts,
                                  skl_info* info);

/* Blendenpik (Avron, Maymounkov and Toledo's solver, the reference's comparison
 * solver): the sketch keeps m = ceil(gamma*d) rows of the randomized DHT of A
 * (random signs D, orthonormal DHT, rows drawn without replacement) instead of
 * hashing them; unpivoted QR of the sample; LSQR preconditioned by R from
 * x = 0; x = R^{-1} y; rank = d.  Uses opts->gamma, it_tol, max_it, wisdom,
 * seed, precision, device and stream; k, use_cpqr, abs_tol and rcond do not
 * apply.  Seeding as the reference's: the signs and the row draw each start
 * from the same reseeded stream (srand(time(NULL)) before each, or opts->seed). */
skl_status skl_dense_blendenpik_solve(const double* A, int64_t lda, int64_t n, int64_t d,
                                      const double* b, double* x, const skl_opts* opts,
                                      skl_info* info);

/* Same with A, b, x in device memory. */
skl_status skl_dense_blendenpik_solve_device(const double* A_dev, int64_t lda, int64_t n,
                                             int64_t d, const double* b_dev, double* x_dev,
                                             const skl_opts* opts, skl_info* info);

/* ------------------------------------------------------- building blocks */

/* The m rows (of N) random_sample keeps, drawn from the library stream
 * (seed_mode/seed as in skl_opts): rows[i], i < m, distinct, in draw order.
 * Bit-exact with select_k_from_n over 0..N-1 for the same stream. */
skl_status skl_subsample_rows(int64_t N, int64_t m, int seed_mode, uint32_t seed, int64_t* rows);

/* Hash rows and values of an m x n s-hashing matrix drawn from the library
 * stream (seed_mode/seed as in skl_opts): rows[i*k+j], vals[i*k+j] =
 * +-1/sqrt(k).  Bit-exact with gen_hashing_matrix for the same stream. */
skl_status skl_hash_generate(int64_t m, int64_t n, int64_t k, int seed_mode, uint32_t seed,
                             int64_t* rows, double* vals);

/* S*A (m x d, column-major, FP32 or FP64 per `precision`, written as double
 * to SA) and S*b for host CSC A and host hash arrays; equilibrate != 0 scales
 * column j of SA by 1/||A(:,j)||_2. */
skl_status skl_sketch_sparse(const skl_csc* A, const double* b, int64_t m, int64_t k,
                             const int64_t* rows, const double* vals, int precision,
                             int equilibrate, double* SA, double* Sb);

/* Orthonormal DHT of the columns of D*A (n x d host, column-major), padded
 * to N rows (N >= n, N even, N/2 a product of 2, 3, 5, 7; zeros below n):
 * Y = H_N [D A; 0] / sqrt(N), computed in FP32 or FP64 per `precision`. */
skl_status skl_dht(const double* A, int64_t lda, int64_t n, int64_t d, const double* D,
                   int64_t N, int precision, double* Y);

/* skl_dht on device buffers without any device allocation.  No counterpart
 * in the reference: it exists for callers that cannot let a library allocate
 * device memory -- a host framework whose caching allocator already owns
 * (nearly) all of the device, code that must keep a fixed device footprint
 * known when the library is loaded, and latency-critical loops where a
 * cudaFree (which synchronises the whole device) would stall other streams.
 *
 * A (lda >= n), D (n entries) and Y (ldy >= N, N x d written) are DEVICE
 * pointers on the current device; the work is enqueued on `stream` (a
 * cudaStream_t; NULL = the legacy default stream) and the call returns
 * without waiting for it.  Results are bit-identical to skl_dht with the same
 * arguments and precision.
 *  - Scratch: one static device array of SKL_DHT_NOALLOC_SCRATCH_BYTES per
 *    device, so N <= SKL_DHT_NOALLOC_MAX_N; a larger N is rejected with
 *    SKL_ERR_INVALID and a message naming the limit.  Nothing in it needs to
 *    start at zero.
 *  - The first call on each device does a one-time set-up (scratch address
 *    lookup, which loads the module holding it, and kernel loading): make that
 *    first call before any stream capture begins.
 *  - All calls on one device share that scratch: calls that may overlap in
 *    time (different streams or host threads without ordering between them)
 *    race on it and give wrong results.  Order them (one stream, or events).
 *  - Footprint: with CUDA's default lazy module loading the array is
 *    committed on a device when this entry point is first used there; with
 *    CUDA_MODULE_LOADING=EAGER, on every device the process initialises.
 *  - After cudaDeviceReset, call skl_finalize() before using it again (the
 *    looked-up address belonged to the destroyed context). */
#define SKL_DHT_NOALLOC_SCRATCH_BYTES (64u << 20)
#define SKL_DHT_NOALLOC_MAX_N 4194304
skl_status skl_dht_device_noalloc(const double* A, int64_t lda, int64_t n, int64_t d,
                                  const double* D, int64_t N, int precision, double* Y,
                                  int64_t ldy, void* stream);

/* Transform length the dense solver uses for n rows (wisdom as in skl_opts). */
int64_t skl_dht_length(int64_t n, int wisdom);

/* alpha*S*(H D A) for the dense path (alpha = 1/sqrt(k), as sketch() applies
 * on top of S's +-1/sqrt(k) values): SA is m x d, Sb is m. */
skl_status skl_sketch_dense(const double* A, int64_t lda, int64_t n, int64_t d,
                            const double* b, const double* D, int64_t N, int64_t m, int64_t k,
                            const int64_t* rows, const double* vals, int precision,
                            double* SA, double* Sb);

/* Randomized column-pivoted QR of the m x d column-major matrix A (host, in
 * place): R in the upper triangle, Householder vectors below, tau[min(m,d)],
 * jpvt[d] 0-based.  precision selects FP32 or FP64 arithmetic. */
skl_status skl_cpqr(double* A, int64_t m, int64_t d, int precision, int64_t* jpvt,
                    double* tau);

/* x <- R^{-1} x (trans = 'n') or R^{-T} x (trans = 't') for the r x r upper
 * triangle of R (column-major, ld), computed on the GPU through the explicit
 * inverse used by the LSQR operator. */
skl_status skl_trsv_upper(const double* R, int64_t ld, int64_t r, char trans, int precision,
                          double* x);

/* y = A x (trans 'n', y has A->m entries) or y = A^T x ('t', A->n entries)
 * through the LSQR product kernels of the solve, with their storage: on the
 * mixed path A's values are equilibrated by column and held as (hi, lo)
 * float pairs with float-float accumulation (relative error of each entry
 * <= 2^-45 of sum_j |a_ij x_j|); on the FP64 path plain FP64.  Replaces the
 * reference's csc_mv (src/SpMat.cpp:37-74) for checking the operator. */
skl_status skl_csc_mv(const skl_csc* A, char trans, const double* x, double* y, int precision);

/* W (b x N, column-major, ld b) = V^T A in FP32 for V (M x b, ldv, b <= 64)
 * and A (M x N, lda), host buffers: the product the randomized CPQR forms
 * for every panel's block reflector.  tensor = 1: the tcgen05 kernel (3xTF32
 * on the tensor cores, TMA-fed, accumulator in tensor memory); tensor = 0:
 * the CUDA-core FP32 kernel.  Each entry is within ~2^-20 of
 * sum_k |v_kc a_kn| of the exact product. */
skl_status skl_gemm_vta(int64_t M, int64_t N, int64_t b, const float* V, int64_t ldv,
                        const float* A, int64_t lda, float* W, int tensor);

/* C (M x N, ldc) rows r0..M-1 -= V Z in FP32, V (M x b, ldv, b <= 64), Z
 * (b x N, ldz), r0 a multiple of 4, host buffers: the randomized CPQR's
 * trailing update of every panel.  tensor = 1: the tcgen05 kernel (3xTF32,
 * TMA loads and stores, accumulator in tensor memory); tensor = 0: the
 * CUDA-core FP32 kernel. */
skl_status skl_gemm_update(int64_t M, int64_t N, int64_t b, int64_t r0, const float* V, int64_t ldv,
                           const float* Z, int64_t ldz, float* C, int64_t ldc, int tensor);

/* Release all device memory and streams held by the library. */
void skl_finalize(void);

#ifdef __cplusplus
}
#endif

#endif /* SKILLS_GB300_H */
