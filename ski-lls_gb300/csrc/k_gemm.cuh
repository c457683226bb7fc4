// k_gemm.cuh -- tiled CUDA-core GEMM for the QR / inverse building blocks.
//
// C = alpha * op(A) * op(B) + beta * C, column-major, op(X) = X or X^T.
// 64x64 output tile per CTA, 256 threads with a 4x4 micro-tile each, K in
// steps of 16 through shared memory.  Split-K writes per-split partials that
// a fixed-order reduction combines (bitwise reproducible).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "skl_internal.hpp"

namespace skl {

constexpr int kGBM = 64, kGBN = 64, kGBK = 16;

// TRI = 0: general.  TRI = 1: op(A) is upper triangular (terms with k < row
// vanish).  TRI = 2: op(B) is upper triangular (terms with k > col vanish).
// Tiles skip the K range that is structurally zero.
template <typename T, bool TA, bool TB, int TRI = 0>
__global__ void __launch_bounds__(256)
k_gemm(int M, int N, int K, T alpha, const T* __restrict__ A, int64_t lda,
       const T* __restrict__ B, int64_t ldb, T beta, T* __restrict__ C, int64_t ldc, int kchunk,
       T* __restrict__ partial)
{
    __shared__ T As[kGBK][kGBM + 1];
    __shared__ T Bs[kGBK][kGBN + 1];
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;     // 16 x 16 threads
    const int m0 = blockIdx.x * kGBM, n0 = blockIdx.y * kGBN;
    int k_begin = blockIdx.z * kchunk;
    int k_end = min(K, k_begin + kchunk);
    if (TRI == 1) k_begin = max(k_begin, m0 / kGBK * kGBK);
    if (TRI == 2) k_end = min(k_end, n0 + kGBN);
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) acc[i][jj] = T(0);

    for (int k0 = k_begin; k0 < k_end; k0 += kGBK) {
        // load op(A)[m0:m0+64, k0:k0+16] -> As[k][m]
#pragma unroll
        for (int e = tid; e < kGBM * kGBK; e += 256) {
            int mm, kk;
            if (!TA) { mm = e % kGBM; kk = e / kGBM; }
            else { kk = e % kGBK; mm = e / kGBK; }
            int gm = m0 + mm, gk = k0 + kk;
            T v = T(0);
            if (gm < M && gk < k_end && (TRI != 1 || gk >= gm))
                v = TA ? A[gk + (int64_t)gm * lda] : A[gm + (int64_t)gk * lda];
            As[kk][mm] = v;
        }
        // load op(B)[k0:k0+16, n0:n0+64] -> Bs[k][n]
#pragma unroll
        for (int e = tid; e < kGBN * kGBK; e += 256) {
            int nn, kk;
            if (!TB) { kk = e % kGBK; nn = e / kGBK; }
            else { nn = e % kGBN; kk = e / kGBN; }
            int gn = n0 + nn, gk = k0 + kk;
            T v = T(0);
            if (gn < N && gk < k_end && (TRI != 2 || gk <= gn))
                v = TB ? B[gn + (int64_t)gk * ldb] : B[gk + (int64_t)gn * ldb];
            Bs[kk][nn] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kGBK; ++kk) {
            T a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][tx + 16 * i];
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) b[jj] = Bs[kk][ty + 16 * jj];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int jj = 0; jj < 4; ++jj) acc[i][jj] = fma(a[i], b[jj], acc[i][jj]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        int gm = m0 + tx + 16 * i;
        if (gm >= M) continue;
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
            int gn = n0 + ty + 16 * jj;
            if (gn >= N) continue;
            if (partial) {
                partial[(int64_t)blockIdx.z * M * N + gm + (int64_t)gn * M] = acc[i][jj];
            } else {
                T* c = C + gm + (int64_t)gn * ldc;
                T v = alpha * acc[i][jj];
                if (beta != T(0)) v += beta * *c;
                *c = v;
            }
        }
    }
}

template <typename T>
__global__ void k_splitk_reduce(int M, int N, int splits, T alpha, const T* __restrict__ partial,
                                T beta, T* __restrict__ C, int64_t ldc)
{
    int64_t total = (int64_t)M * N;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        T s = T(0);
        for (int z = 0; z < splits; ++z) s += partial[(int64_t)z * total + e];
        int gm = (int)(e % M);
        int64_t gn = e / M;
        T* c = C + gm + gn * ldc;
        T v = alpha * s;
        if (beta != T(0)) v += beta * *c;
        *c = v;
    }
}

// Picks a split-K factor so that the grid covers the GPU when the output is
// small and K is long.  partial must hold splits*M*N entries when splits > 1.
inline int gemm_splits(int M, int N, int K)
{
    int tiles = ((M + kGBM - 1) / kGBM) * ((N + kGBN - 1) / kGBN);
    int s = 1;
    while (tiles * s < 2 * 152 && K / (s * 2) >= 256 && s < 32) s *= 2;
    return s;
}

template <typename T>
void gemm(bool ta, bool tb, int M, int N, int K, T alpha, const T* A, int64_t lda, const T* B,
          int64_t ldb, T beta, T* C, int64_t ldc, T* partial, int64_t partial_cap,
          cudaStream_t st)
{
    if (M <= 0 || N <= 0) return;
    int splits = (K > 0 && partial) ? gemm_splits(M, N, K) : 1;
    while (splits > 1 && (int64_t)splits * M * N > partial_cap) splits >>= 1;
    int kchunk = K;
    if (splits > 1) {
        kchunk = (K + splits - 1) / splits;
        kchunk = (kchunk + kGBK - 1) / kGBK * kGBK;
        splits = (K + kchunk - 1) / kchunk;
    }
    if (K <= 0) { kchunk = 0; splits = 1; }
    dim3 grid((M + kGBM - 1) / kGBM, (N + kGBN - 1) / kGBN, splits);
    T* part = splits > 1 ? partial : nullptr;
    if (!ta && !tb) k_gemm<T, false, false><<<grid, 256, 0, st>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, kchunk, part);
    else if (ta && !tb) k_gemm<T, true, false><<<grid, 256, 0, st>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, kchunk, part);
    else if (!ta && tb) k_gemm<T, false, true><<<grid, 256, 0, st>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, kchunk, part);
    else k_gemm<T, true, true><<<grid, 256, 0, st>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, kchunk, part);
    SKL_LAUNCHED();
    if (splits > 1) {
        int64_t total = (int64_t)M * N;
        unsigned g = (unsigned)((total + 255) / 256);
        if (g > 152 * 8) g = 152 * 8;
        k_splitk_reduce<T><<<g, 256, 0, st>>>(M, N, splits, alpha, partial, beta, C, ldc);
        SKL_LAUNCHED();
    }
}

// C = alpha * A * B + beta * C with A upper triangular (tri = 1) or B upper
// triangular (tri = 2); no transposes, no split-K.
template <typename T>
void trmm(int tri, int M, int N, int K, T alpha, const T* A, int64_t lda, const T* B, int64_t ldb,
          T beta, T* C, int64_t ldc, cudaStream_t st)
{
    if (M <= 0 || N <= 0) return;
    dim3 grid((M + kGBM - 1) / kGBM, (N + kGBN - 1) / kGBN, 1);
    if (tri == 1)
        k_gemm<T, false, false, 1><<<grid, 256, 0, st>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, K, nullptr);
    else
        k_gemm<T, false, false, 2><<<grid, 256, 0, st>>>(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, K, nullptr);
    SKL_LAUNCHED();
}

}  // namespace skl
