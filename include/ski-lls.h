/*
 * ski-lls.h -- C++ drop-in for the Ski-LLS solver entry points, running on a
 * GB300 GPU through the C ABI of skills_gb300.h.
 *
 * Keeps the three signatures of the reference's include/ski-lls.h:15-28
 * (ls_dense_hashing_blendenpik, ls_dense_hashing_blendenpik_noCPQR,
 * ls_sparse_spqr), the solver defaults of include/bench_config.hpp:7-20, and the
 * small part of the container API its example programs use (Mat_d, Vec_d, a
 * cs_dl with CSparse's field layout, CSC_Mat_d::mv, nrm2, operator<<), so a
 * program written against the reference builds unchanged when it includes this
 * header instead and links libskills_gb300.so.  Errors are thrown as
 * std::runtime_error with the reference's messages.
 *
 * Differences a caller can observe: A is left untouched by the dense solver
 * (the reference permutes it in place and restores it); the sketch factorization
 * is a GPU randomized CPQR, so R, the pivots and, on rank-deficient input, the
 * basic solution can differ from SuiteSparseQR's while the residual agrees.
 */
#ifndef SKILLS_H
#define SKILLS_H

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <memory>
#include <stdexcept>
#include <string>

#include "skills_gb300.h"

/* include/bench_config.hpp:7-20 */
#define IT_TOL 1e-6
#define MAX_IT 10000
#define OVER_SAMPLING_RATIO 1.1
#define NNZ_PER_COLUMN 3
#define PERTURB 1e-10
#define RCOND_THRESHOLD 1e-10
#define ORDERING 0
#define SCALING 0
#define SHIFTING 1e-12
#define RCOND 1e-10
#define WISDOM 0
#define PRINTING_PRECISION 17
#define ABS_TOL 1e-8
#define SPQR_ORDERING 2

/* include/ski-lls.h:11-12 */
#define FFTW_R2R_DCT 1
#define FFTW_R2R_DHT 2

/* ------------------------------------------------------------ containers -- */

/* Strided vector over owned or borrowed storage (reference: include/Vec.hpp). */
template <typename T>
class Vec {
public:
    typedef long idx_t;
    Vec(idx_t n = 0) : n_(n), inc_(1), own_(n > 0 ? new T[(size_t)n]() : nullptr, std::default_delete<T[]>())
    {
        data_ = own_.get();
    }
    Vec(idx_t n, T* data, idx_t inc = 1) : n_(n), inc_(inc), data_(data) {}
    idx_t const& n() const { return n_; }
    idx_t const& inc() const { return inc_; }
    T* data() const { return data_; }
    T& operator()(idx_t i) const { return data_[i * inc_]; }
    Vec copy() const
    {
        Vec v(n_);
        for (idx_t i = 0; i < n_; ++i) v(i) = (*this)(i);
        return v;
    }

private:
    idx_t n_, inc_;
    std::shared_ptr<T> own_;
    T* data_ = nullptr;
};

/* Column-major matrix with leading dimension (reference: include/Mat.hpp). */
template <typename T>
class Mat {
public:
    typedef long idx_t;
    Mat(idx_t m = 0, idx_t n = 0, idx_t ld = -1)
        : m_(m), n_(n), ld_(ld < 0 ? m : ld),
          own_(m * n > 0 ? new T[(size_t)((ld < 0 ? m : ld) * n)]() : nullptr, std::default_delete<T[]>())
    {
        data_ = own_.get();
    }
    Mat(idx_t m, idx_t n, T* data, idx_t ld = -1) : m_(m), n_(n), ld_(ld < 0 ? m : ld), data_(data) {}
    idx_t const& m() const { return m_; }
    idx_t const& n() const { return n_; }
    idx_t const& ld() const { return ld_; }
    T* data() const { return data_; }
    T& operator()(idx_t i, idx_t j) const { return data_[i + j * ld_]; }
    /* y = alpha*op(A)*x + beta*y, op = 'n' or 't' (dgemv semantics) */
    void mv(const char trans, const T alpha, const Vec<T>& x, const T beta, Vec<T>& y) const
    {
        if (trans == 'n') {
            for (idx_t i = 0; i < m_; ++i) y(i) = beta == T(0) ? T(0) : beta * y(i);
            for (idx_t j = 0; j < n_; ++j) {
                const T t = alpha * x(j);
                for (idx_t i = 0; i < m_; ++i) y(i) += t * (*this)(i, j);
            }
        } else if (trans == 't') {
            for (idx_t j = 0; j < n_; ++j) {
                T s = T(0);
                for (idx_t i = 0; i < m_; ++i) s += (*this)(i, j) * x(i);
                y(j) = (beta == T(0) ? T(0) : beta * y(j)) + alpha * s;
            }
        } else {
            throw std::runtime_error("trans must be either 'n' or 't'.");
        }
    }

private:
    idx_t m_, n_, ld_;
    std::shared_ptr<T> own_;
    T* data_ = nullptr;
};

typedef Vec<double> Vec_d;
typedef Mat<double> Mat_d;

template <typename T>
inline T nrm2(const Vec<T>& x)
{
    long double s = 0;
    for (long i = 0; i < x.n(); ++i) s += (long double)x(i) * x(i);
    return (T)std::sqrt(s);
}

template <typename T>
inline std::ostream& operator<<(std::ostream& os, const Vec<T>& v)
{
    for (long i = 0; i < v.n(); ++i) os << v(i) << (i + 1 < v.n() ? " " : "");
    return os;
}

template <typename T>
inline std::ostream& operator<<(std::ostream& os, const Mat<T>& A)
{
    for (long i = 0; i < A.m(); ++i) {
        for (long j = 0; j < A.n(); ++j) os << A(i, j) << (j + 1 < A.n() ? " " : "");
        os << "\n";
    }
    return os;
}

/* CSparse's cs_dl layout (64-bit indices), as the reference's callers build it
 * with cs_dl_spalloc and then overwrite p, i, x (test/ski-llsSparseExample.cpp:15-20). */
typedef struct cs_dl_sparse {
    int64_t nzmax;
    int64_t m;
    int64_t n;
    int64_t* p;
    int64_t* i;
    double* x;
    int64_t nz;   /* -1 for compressed-column form */
} cs_dl;

inline cs_dl* cs_dl_spalloc(int64_t m, int64_t n, int64_t nzmax, int64_t values, int64_t triplet)
{
    cs_dl* A = (cs_dl*)std::calloc(1, sizeof(cs_dl));
    if (!A) return nullptr;
    A->m = m;
    A->n = n;
    A->nzmax = nzmax > 1 ? nzmax : 1;
    A->nz = triplet ? 0 : -1;
    A->p = (int64_t*)std::calloc((size_t)(triplet ? A->nzmax : n + 1), sizeof(int64_t));
    A->i = (int64_t*)std::calloc((size_t)A->nzmax, sizeof(int64_t));
    A->x = values ? (double*)std::calloc((size_t)A->nzmax, sizeof(double)) : nullptr;
    return A;
}

/* Prints the matrix dimensions and, when brief == 0, its columns. */
inline int64_t cs_dl_print(const cs_dl* A, int64_t brief)
{
    if (!A) {
        std::printf("(null)\n");
        return 0;
    }
    const int64_t nnz = A->nz < 0 ? A->p[A->n] : A->nz;
    std::printf("%lld-by-%lld, nzmax: %lld nnz: %lld\n", (long long)A->m, (long long)A->n,
                (long long)A->nzmax, (long long)nnz);
    if (brief || A->nz >= 0) return 1;
    for (int64_t j = 0; j < A->n; ++j) {
        std::printf("    col %lld : locations %lld to %lld\n", (long long)j, (long long)A->p[j],
                    (long long)(A->p[j + 1] - 1));
        for (int64_t q = A->p[j]; q < A->p[j + 1]; ++q)
            std::printf("      %lld : %g\n", (long long)A->i[q], A->x ? A->x[q] : 1.0);
    }
    return 1;
}

/* Compressed-column view (reference: include/SpMat.hpp CSC_Mat): constructed
 * as CSC_Mat_d(m, n, nnz, row_indices, col_ptr, values). */
template <typename T>
class CSC_Mat {
public:
    typedef long idx_t;
    CSC_Mat(idx_t m, idx_t n, idx_t nnz, long* ir, long* jc, T* data)
        : m_(m), n_(n), nnz_(nnz), ir_(ir), jc_(jc), data_(data) {}
    idx_t const& m() const { return m_; }
    idx_t const& n() const { return n_; }
    /* y = alpha*op(A)*x + beta*y (src/SpMat.cpp:37-74 semantics) */
    void mv(const char trans, const T alpha, const Vec<T>& x, const T beta, Vec<T>& y) const
    {
        if (trans == 'n') {
            for (idx_t i = 0; i < m_; ++i) y(i) = beta == T(0) ? T(0) : beta * y(i);
            for (idx_t j = 0; j < n_; ++j)
                for (idx_t q = jc_[j]; q < jc_[j + 1]; ++q) y(ir_[q]) += alpha * data_[q] * x(j);
        } else if (trans == 't') {
            for (idx_t j = 0; j < n_; ++j) y(j) = beta == T(0) ? T(0) : beta * y(j);
            for (idx_t j = 0; j < n_; ++j)
                for (idx_t q = jc_[j]; q < jc_[j + 1]; ++q) y(j) += alpha * data_[q] * x(ir_[q]);
        } else {
            throw std::runtime_error("trans must be either 'n' or 't'.");
        }
    }

private:
    idx_t m_, n_, nnz_;
    long* ir_;
    long* jc_;
    T* data_;
};
typedef CSC_Mat<double> CSC_Mat_d;

/* ------------------------------------------------------------ solvers ----- */

namespace skills_gb300_detail {
inline void check(skl_status s)
{
    if (s != SKL_OK) throw std::runtime_error(skl_last_error());
}
}  // namespace skills_gb300_detail

/* ls_dense_hashing_blendenpik (include/ski-lls.h:15-17): sign + DHT + hash
 * sketch, randomized CPQR with the absolute |R_ii| > rcond rank rule, LSQR
 * preconditioned by R11 from the sketch solution.  The sign/hash stream is
 * seeded with time(NULL), as the reference does. */
inline void ls_dense_hashing_blendenpik(Mat_d& A, Vec_d& b, Vec_d& x, long& rank, int& flag,
                                        long& it, double gamma, long k, double abs_tol,
                                        double rcond, double it_tol, long max_it, int debug,
                                        int wisdom)
{
    (void)debug;
    if (A.m() != b.n() || A.n() != x.n() || b.inc() != 1 || x.inc() != 1)
        throw std::runtime_error("size mismatch");
    skl_opts o;
    skl_default_opts(&o);
    o.gamma = gamma;
    o.k = k;
    o.abs_tol = abs_tol;
    o.rcond = rcond;
    o.it_tol = it_tol;
    o.max_it = max_it;
    o.wisdom = wisdom;
    o.use_cpqr = 1;
    skl_info info;
    skills_gb300_detail::check(skl_dense_solve(A.data(), A.ld(), A.m(), A.n(), b.data(), x.data(), &o, &info));
    rank = (long)info.rank;
    flag = info.flag;
    it = (long)info.it;
}

/* ls_dense_hashing_blendenpik_noCPQR (include/ski-lls.h:19-21): unpivoted QR
 * of the sketch, LSQR from zero, rank = n. */
inline void ls_dense_hashing_blendenpik_noCPQR(Mat_d& A, Vec_d& b, Vec_d& x, long& rank, int& flag,
                                               long& it, double gamma, long k, double it_tol,
                                               long max_it, int debug, int wisdom)
{
    (void)debug;
    if (A.m() != b.n() || A.n() != x.n() || b.inc() != 1 || x.inc() != 1)
        throw std::runtime_error("size mismatch");
    skl_opts o;
    skl_default_opts(&o);
    o.gamma = gamma;
    o.k = k;
    o.it_tol = it_tol;
    o.max_it = max_it;
    o.wisdom = wisdom;
    o.use_cpqr = 0;
    o.abs_tol = 0.0;
    skl_info info;
    skills_gb300_detail::check(skl_dense_solve(A.data(), A.ld(), A.m(), A.n(), b.data(), x.data(), &o, &info));
    rank = (long)info.rank;
    flag = info.flag;
    it = (long)info.it;
}

/* ls_sparse_spqr (include/ski-lls.h:24-28): s-hashing sketch drawn from the
 * library's C-library-compatible random stream (a fresh process starts at seed
 * 1, like rand()), randomized CPQR of the sketch, R11 condition test with pivot
 * perturbation, LSQR preconditioned by R11.  `ordering` is accepted for
 * signature compatibility. */
inline void ls_sparse_spqr(cs_dl& A, Vec_d& b, Vec_d& x, long& rank, int& flag, long& it,
                           double gamma, long k, double abs_tol = ABS_TOL,
                           int ordering = SPQR_ORDERING, double it_tol = IT_TOL,
                           long max_it = MAX_IT, double rcond_threshold = RCOND_THRESHOLD,
                           double perturb = PERTURB, int debug = 0)
{
    (void)ordering;
    (void)debug;
    if (A.m != b.n() || A.n != x.n() || b.inc() != 1 || x.inc() != 1)
        throw std::runtime_error("size mismatch");
    skl_opts o;
    skl_default_opts(&o);
    o.gamma = gamma;
    o.k = k;
    o.abs_tol = abs_tol;
    o.it_tol = it_tol;
    o.max_it = max_it;
    o.rcond_threshold = rcond_threshold;
    o.perturb = perturb;
    skl_csc csc;
    csc.m = A.m;
    csc.n = A.n;
    csc.nzmax = A.nzmax;
    csc.p = A.p;
    csc.i = A.i;
    csc.x = A.x;
    skl_info info;
    skills_gb300_detail::check(skl_sparse_solve(&csc, b.data(), x.data(), &o, &info));
    rank = (long)info.rank;
    flag = info.flag;
    it = (long)info.it;
}

#endif /* SKILLS_H */
