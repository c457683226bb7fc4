// k_trinv.cu -- explicit inverse of the triangular preconditioner R11, rank
// detection and the condition estimate.
//
// The reference applies R11^{-1} by substitution twice per LSQR iteration
// (cs_usolve/cs_utsolve_cholmod_structure, src/sparse_helpers.cpp:122-181;
// dtrsv in LinOP_dense_preconditioner, src/IterSolver.cpp:84-99).  On a GPU a
// substitution is a chain of d dependent steps; here M = R11^{-1} is formed
// once (d^3/3 flops) so that each application is a bandwidth-bound triangular
// mat-vec.  LSQR then runs on the operator A*P1*D*M, which is exactly
// A*P1*R11^{-1} up to the rounding of M; the same M is used for the forward
// and the transposed products, so the iteration stays consistent.
//
// The condition test of rnpre_sparse (dtrcon 'I' on R11 vs rcond_threshold,
// src/ls_sparse_spqr.cpp:64-69, src/cholmod_cond_est.cpp:12-34) uses the
// exact 1/(||R11||_inf ||R11^{-1}||_inf) available from M.
#include <cmath>

#include "skl_internal.hpp"
#include "launch.cuh"
#include "common.cuh"
#include "k_gemm.cuh"

namespace skl {

constexpr int kTB = 64;   // diagonal block size
constexpr int kBatchMaxBlock = 512;   // levels up to this block size run as one batched launch per product

// Invert the 64x64 (or smaller, last) diagonal blocks of R (+ perturb*I):
// one CTA per block, one thread per column of the inverse.
template <typename T>
__global__ void k_inv_diag_blocks(const T* __restrict__ R, int64_t ld, int r, T perturb,
                                  T* __restrict__ M, int64_t ldm)
{
    pdl_wait();
    __shared__ T U[kTB][kTB + 1];
    __shared__ T X[kTB][kTB + 1];
    const int b0 = blockIdx.x * kTB;
    const int bs = min(kTB, r - b0);
    for (int e = threadIdx.x; e < kTB * kTB; e += blockDim.x) {
        int i = e % kTB, j = e / kTB;
        T v = T(0);
        if (i < bs && j < bs && i <= j) v = R[(b0 + i) + (int64_t)(b0 + j) * ld];
        if (i == j && i < bs) v += perturb;
        U[i][j] = v;
        X[i][j] = T(0);
    }
    __syncthreads();
    const int c = threadIdx.x;
    if (c < bs) {
        // column c of U^{-1}: back substitution
        X[c][c] = T(1) / U[c][c];
        for (int i = c - 1; i >= 0; --i) {
            T acc = T(0);
            for (int k = i + 1; k <= c; ++k) acc += U[i][k] * X[k][c];
            X[i][c] = -acc / U[i][i];
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < kTB * kTB; e += blockDim.x) {
        int i = e % kTB, j = e / kTB;
        if (i < bs && j < bs) M[(b0 + i) + (int64_t)(b0 + j) * ldm] = X[i][j];
    }
}

template <typename T>
__global__ void k_zero_lower(T* __restrict__ M, int64_t ldm, int r)
{
    pdl_wait();
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)r * r;
         e += (int64_t)gridDim.x * blockDim.x) {
        int i = (int)(e % r);
        int j = (int)(e / r);
        if (i > j && (i / kTB) != (j / kTB)) M[i + (int64_t)j * ldm] = T(0);
    }
}

template <typename T>
size_t trinv_workspace_bytes(int64_t r)
{
    // B C^{-1} of one pair (at most r^2 / 4) and the split-K partials of the
    // pair's two products behind it
    const size_t a = (size_t)r * r * sizeof(T) + (size_t)kTB * kTB * sizeof(T);
    const size_t b = (size_t)((r + 127) / 128) * r * sizeof(double);   // row-sum partials
    return (a > b ? a : b) + 4096;
}

// ||upper triangle||_inf: row sums of |X| accumulated per (row block, column
// chunk) tile in fixed order, then the max over rows.  FP64 sums.
constexpr int kInfRows = 128, kInfCols = 128;
template <typename T>
__global__ void k_inf_rowsum_tiles(const T* __restrict__ X, int64_t ld, int r, double* __restrict__ part)
{
    pdl_wait();
    const int i = blockIdx.x * kInfRows + threadIdx.x;
    const int j0 = blockIdx.y * kInfCols;
    double s = 0.0;
    if (i < r) {
        const int jb = max(i, j0), je = min(r, j0 + kInfCols);
        for (int j = jb; j < je; ++j) s += fabs((double)X[i + (int64_t)j * ld]);
    }
    if (i < r) part[(int64_t)blockIdx.y * r + i] = s;
}

__global__ void k_inf_rowsum_max(const double* __restrict__ part, int nchunks, int r, double* out)
{
    pdl_wait();
    __shared__ double red[32];
    double mx = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < r; i += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int q = 0; q < nchunks; ++q) s += part[(int64_t)q * r + i];
        mx = s > mx ? s : mx;
    }
    mx = block_max(mx, red);
    if (threadIdx.x == 0) atomicMax((unsigned long long*)out, (unsigned long long)__double_as_longlong(mx));
}

template <typename T>
static void inf_norm_upper(const T* X, int64_t ld, int64_t r, double* part, double* out, cudaStream_t st)
{
    const int nchunks = (int)((r + kInfCols - 1) / kInfCols);
    dim3 g((unsigned)((r + kInfRows - 1) / kInfRows), nchunks);
    launch_k(k_inf_rowsum_tiles<T>, g, kInfRows, 0, st, X, ld, (int)r, part);
    launch_k(k_inf_rowsum_max, (unsigned)std::min<int64_t>((r + 255) / 256, 64), 256, 0, st, part, nchunks, (int)r, out);
    SKL_LAUNCHED();
    SKL_LAUNCHED();
}

template <typename T>
void trinv_upper(const T* R, int64_t ld, int64_t r, double perturb, T* M, int64_t ldm,
                 double* norms, void* work, cudaStream_t st)
{
    if (r <= 0) return;
    const int nblk = (int)((r + kTB - 1) / kTB);
    launch_k(k_inv_diag_blocks<T>, nblk, kTB, 0, st, R, ld, (int)r, (T)perturb, M, ldm);
    SKL_LAUNCHED();
    T* tmp = (T*)work;   // holds B * C^{-1} for one pair (s x s')
    const size_t ws_elems = (trinv_workspace_bytes<T>(r) - 4096) / sizeof(T);
    // recursive doubling: blocks of size s are inverted; combine neighbours
    for (int64_t s = kTB; s < r; s *= 2) {
        int64_t a_first = 0;
        if (s <= kBatchMaxBlock) {
            // all full pairs of this level in two launches
            const int64_t full = r / (2 * s);
            if (full > 0) {
                const int64_t step = 2 * s * (ldm + 1);
                trmm_batched<T>(2, (int)s, (int)s, (int)s, T(1), R + s * ld, ld, 2 * s * (ld + 1),
                                M + s + s * ldm, ldm, step, T(0), tmp, s, s * s, (int)full, st);
                trmm_batched<T>(1, (int)s, (int)s, (int)s, T(-1), M, ldm, step, tmp, s, s * s, T(0),
                                M + s * ldm, ldm, step, (int)full, st);
                a_first = full * 2 * s;
            }
        }
        for (int64_t a0 = a_first; a0 + s < r; a0 += 2 * s) {
            const int64_t c0 = a0 + s;
            const int64_t sa = s;
            const int64_t sc = std::min<int64_t>(s, r - c0);
            const T* Ainv = M + a0 + a0 * ldm;
            const T* Cinv = M + c0 + c0 * ldm;
            const T* Bblk = R + a0 + c0 * ld;
            T* X = M + a0 + c0 * ldm;
            // tmp = B * Cinv (Cinv upper), then X = -Ainv * tmp (Ainv upper);
            // the K-split partials sit behind tmp (FP32 products only)
            T* part = tmp + (sa * sc + 3) / 4 * 4;
            const int64_t cap = (int64_t)(ws_elems - (size_t)(part - tmp));
            trmm<T>(2, (int)sa, (int)sc, (int)sc, T(1), Bblk, ld, Cinv, ldm, T(0), tmp, sa, st, part, cap);
            trmm<T>(1, (int)sa, (int)sc, (int)sa, T(-1), Ainv, ldm, tmp, sa, T(0), X, ldm, st, part, cap);
        }
    }
    launch_k(k_zero_lower<T>, 1024, 256, 0, st, M, ldm, (int)r);
    SKL_LAUNCHED();
    cudaMemsetAsync(norms, 0, 2 * sizeof(double), st);
    // row-sum partials reuse the inverse's scratch (free again here)
    double* part = (double*)work;
    inf_norm_upper<T>(R, ld, r, part, norms, st);
    inf_norm_upper<T>(M, ldm, r, part, norms + 1, st);
}

// Number of leading diagonal entries with |R_ii| > max(abs_thresh, rel_thresh*|R_00|).
template <typename T>
__global__ void k_rank(const T* __restrict__ R, int64_t ld, int dmin, double abs_thresh,
                       double rel_thresh, int* out)
{
    pdl_wait();
    __shared__ int red[32];
    const double r00 = dmin > 0 ? fabs((double)R[0]) : 0.0;
    const double th = fmax(abs_thresh, rel_thresh * r00);
    int first = dmin;
    for (int i = threadIdx.x; i < dmin; i += blockDim.x) {
        double v = fabs((double)R[i + (int64_t)i * ld]);
        if (!(v > th) && i < first) first = i;
    }
    // block min
    for (int o = 16; o > 0; o >>= 1) {
        int w = __shfl_xor_sync(0xffffffffu, first, o);
        first = w < first ? w : first;
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = first;
    __syncthreads();
    if (threadIdx.x == 0) {
        int f = dmin;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) f = red[w] < f ? red[w] : f;
        *out = f;
    }
}

template <typename T>
int64_t count_rank(const T* R, int64_t ld, int64_t dmin, double abs_thresh, double rel_thresh,
                   int* dev_out, int* host_pinned, cudaStream_t st)
{
    launch_k(k_rank<T>, 1, 1024, 0, st, R, ld, (int)dmin, abs_thresh, rel_thresh, dev_out);
    SKL_LAUNCHED();
    SKL_CUDA(cudaMemcpyAsync(host_pinned, dev_out, sizeof(int), cudaMemcpyDeviceToHost, st));
    SKL_CUDA(cudaStreamSynchronize(st));
    return *host_pinned;
}

template size_t trinv_workspace_bytes<float>(int64_t);
template size_t trinv_workspace_bytes<double>(int64_t);
template void trinv_upper<float>(const float*, int64_t, int64_t, double, float*, int64_t, double*,
                                 void*, cudaStream_t);
template void trinv_upper<double>(const double*, int64_t, int64_t, double, double*, int64_t,
                                  double*, void*, cudaStream_t);
template int64_t count_rank<float>(const float*, int64_t, int64_t, double, double, int*, int*,
                                   cudaStream_t);
template int64_t count_rank<double>(const double*, int64_t, int64_t, double, double, int*, int*,
                                    cudaStream_t);

}  // namespace skl

namespace skl {

// y = M x (trans 'n') or M^T x (trans 't') for the r x r upper triangle of M,
// FP64 accumulation; one thread per output entry (building-block API only).
template <typename T>
__global__ void k_trmv_upper(const T* __restrict__ M, int64_t ldm, int r, int trans,
                             const double* __restrict__ x, double* __restrict__ y)
{
    pdl_wait();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < r; i += gridDim.x * blockDim.x) {
        double acc = 0.0;
        if (!trans)
            for (int j = i; j < r; ++j) acc = fma((double)M[i + (int64_t)j * ldm], x[j], acc);
        else
            for (int j = 0; j <= i; ++j) acc = fma((double)M[j + (int64_t)i * ldm], x[j], acc);
        y[i] = acc;
    }
}

template <typename T>
void trmv_upper(const T* M, int64_t ldm, int64_t r, int trans, const double* x, double* y,
                cudaStream_t st)
{
    if (r <= 0) return;
    launch_k(k_trmv_upper<T>, (unsigned)((r + 127) / 128), 128, 0, st, M, ldm, (int)r, trans, x, y);
    SKL_LAUNCHED();
}
template void trmv_upper<float>(const float*, int64_t, int64_t, int, const double*, double*,
                                cudaStream_t);
template void trmv_upper<double>(const double*, int64_t, int64_t, int, const double*, double*,
                                 cudaStream_t);

}  // namespace skl
