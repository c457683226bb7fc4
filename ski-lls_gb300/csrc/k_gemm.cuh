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
#include "launch.cuh"

namespace skl {

constexpr int kGBM = 64, kGBN = 64, kGBK = 16;

// TRI = 0: general.  TRI = 1: op(A) is upper triangular (terms with k < row
// vanish).  TRI = 2: op(B) is upper triangular (terms with k > col vanish).
// Tiles skip the K range that is structurally zero.
// BAT: blockIdx.z indexes a batch of equally shaped products whose operands
// sit bsa / bsb / bsc elements apart (no split-K).
template <typename T, bool TA, bool TB, int TRI = 0, bool BAT = false>
__global__ void __launch_bounds__(256)
k_gemm(int M, int N, int K, T alpha, const T* __restrict__ A, int64_t lda,
       const T* __restrict__ B, int64_t ldb, T beta, T* __restrict__ C, int64_t ldc, int kchunk,
       T* __restrict__ partial, int64_t bsa = 0, int64_t bsb = 0, int64_t bsc = 0)
{
    pdl_wait();
    __shared__ T As[kGBK][kGBM + 1];
    __shared__ T Bs[kGBK][kGBN + 1];
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;     // 16 x 16 threads
    const int m0 = blockIdx.x * kGBM, n0 = blockIdx.y * kGBN;
    if (BAT) {
        A += blockIdx.z * bsa;
        B += blockIdx.z * bsb;
        C += blockIdx.z * bsc;
        partial = nullptr;
    }
    int k_begin = BAT ? 0 : blockIdx.z * kchunk;
    int k_end = BAT ? K : min(K, k_begin + kchunk);
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

// ---------------------------------------------------------------- FP32 ----
// Register-prefetched, double-buffered FP32 GEMM: 128 x 128 (MT = 2) or
// 64 x 128 (MT = 1) output tile per 256-thread CTA, K in steps of 8, each
// thread an 8 x 8 (4 x 8) micro-tile read as float4 from padded shared
// memory.  Global loads are float4 where the tile edge and the alignment
// allow, scalar otherwise; the next K step's loads are in flight while the
// current one is multiplied.  Same contract as k_gemm (TRI, split-K).
constexpr int kSBN = 128, kSBK = 8, kSPad = 4;

template <int MT, bool TA, int TRI>
SKL_DEV void sgemm_load_a(const float* __restrict__ A, int64_t lda, int M, int m0, int k0, int k_end,
                          bool vec, float4 (&ra)[1], int tid)
{
    constexpr int BM = 64 * MT;
    constexpr int NCH = BM * kSBK / 4;   // float4 chunks in the tile
    if (tid >= NCH) return;
    const int c = tid;
    float v[4];
    if (!TA) {
        const int k = c / (BM / 4), m4 = (c % (BM / 4)) * 4;
        const int gm = m0 + m4, gk = k0 + k;
        // a triangular operand still loads whole float4s away from its diagonal
        if (vec && gk < k_end && gm + 3 < M && (TRI != 1 || gk >= gm + 3)) {
            ra[0] = *reinterpret_cast<const float4*>(A + gm + (int64_t)gk * lda);
            return;
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int mm = gm + q;
            v[q] = (mm < M && gk < k_end && (TRI != 1 || gk >= mm)) ? A[mm + (int64_t)gk * lda] : 0.f;
        }
    } else {
        const int m = c / (kSBK / 4), k4 = (c % (kSBK / 4)) * 4;
        const int gm = m0 + m, gk = k0 + k4;
        if (vec && gm < M && gk + 3 < k_end && (TRI != 1 || gk >= gm)) {
            ra[0] = *reinterpret_cast<const float4*>(A + gk + (int64_t)gm * lda);
            return;
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int kk = gk + q;
            v[q] = (gm < M && kk < k_end && (TRI != 1 || kk >= gm)) ? A[kk + (int64_t)gm * lda] : 0.f;
        }
    }
    ra[0] = make_float4(v[0], v[1], v[2], v[3]);
}

template <int MT, bool TA>
SKL_DEV void sgemm_store_a(float (*As)[64 * MT + kSPad], const float4 (&ra)[1], int tid)
{
    constexpr int BM = 64 * MT;
    constexpr int NCH = BM * kSBK / 4;
    if (tid >= NCH) return;
    const int c = tid;
    if (!TA) {
        const int k = c / (BM / 4), m4 = (c % (BM / 4)) * 4;
        *reinterpret_cast<float4*>(&As[k][m4]) = ra[0];
    } else {
        const int m = c / (kSBK / 4), k4 = (c % (kSBK / 4)) * 4;
        As[k4 + 0][m] = ra[0].x;
        As[k4 + 1][m] = ra[0].y;
        As[k4 + 2][m] = ra[0].z;
        As[k4 + 3][m] = ra[0].w;
    }
}

template <bool TB, int TRI>
SKL_DEV void sgemm_load_b(const float* __restrict__ B, int64_t ldb, int N, int n0, int k0, int k_end,
                          bool vec, float4 (&rb)[1], int tid)
{
    const int c = tid;   // kSBN * kSBK / 4 == 256 chunks
    float v[4];
    if (!TB) {
        const int n = c / (kSBK / 4), k4 = (c % (kSBK / 4)) * 4;
        const int gn = n0 + n, gk = k0 + k4;
        if (vec && gn < N && gk + 3 < k_end && (TRI != 2 || gk + 3 <= gn)) {
            rb[0] = *reinterpret_cast<const float4*>(B + gk + (int64_t)gn * ldb);
            return;
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int kk = gk + q;
            v[q] = (gn < N && kk < k_end && (TRI != 2 || kk <= gn)) ? B[kk + (int64_t)gn * ldb] : 0.f;
        }
    } else {
        const int k = c / (kSBN / 4), n4 = (c % (kSBN / 4)) * 4;
        const int gn = n0 + n4, gk = k0 + k;
        if (vec && gk < k_end && gn + 3 < N && (TRI != 2 || gk <= gn)) {
            rb[0] = *reinterpret_cast<const float4*>(B + gn + (int64_t)gk * ldb);
            return;
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int nn = gn + q;
            v[q] = (nn < N && gk < k_end && (TRI != 2 || gk <= nn)) ? B[nn + (int64_t)gk * ldb] : 0.f;
        }
    }
    rb[0] = make_float4(v[0], v[1], v[2], v[3]);
}

template <bool TB>
SKL_DEV void sgemm_store_b(float (*Bs)[kSBN + kSPad], const float4 (&rb)[1], int tid)
{
    const int c = tid;
    if (!TB) {
        const int n = c / (kSBK / 4), k4 = (c % (kSBK / 4)) * 4;
        Bs[k4 + 0][n] = rb[0].x;
        Bs[k4 + 1][n] = rb[0].y;
        Bs[k4 + 2][n] = rb[0].z;
        Bs[k4 + 3][n] = rb[0].w;
    } else {
        const int k = c / (kSBN / 4), n4 = (c % (kSBN / 4)) * 4;
        *reinterpret_cast<float4*>(&Bs[k][n4]) = rb[0];
    }
}

template <int MT, bool TA, bool TB, int TRI>
__global__ void __launch_bounds__(256, 2)
k_sgemm(int M, int N, int K, float alpha, const float* __restrict__ A, int64_t lda,
        const float* __restrict__ B, int64_t ldb, float beta, float* __restrict__ C, int64_t ldc,
        int kchunk, float* __restrict__ partial)
{
    pdl_wait();
    constexpr int BM = 64 * MT;
    __shared__ __align__(16) float As[2][kSBK][BM + kSPad];
    __shared__ __align__(16) float Bs[2][kSBK][kSBN + kSPad];
    const int tid = threadIdx.x;
    const int tm = tid & 15, tn = tid >> 4;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * kSBN;
    int k_begin = blockIdx.z * kchunk;
    int k_end = min(K, k_begin + kchunk);
    if (TRI == 1) k_begin = max(k_begin, m0 / kSBK * kSBK);
    if (TRI == 2) k_end = min(k_end, n0 + kSBN);
    const bool veca = ((reinterpret_cast<uintptr_t>(A) & 15) == 0) && (lda & 3) == 0;
    const bool vecb = ((reinterpret_cast<uintptr_t>(B) & 15) == 0) && (ldb & 3) == 0;

    float acc[4 * MT][8];
#pragma unroll
    for (int i = 0; i < 4 * MT; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;

    float4 ra[1], rb[1];
    if (k_begin < k_end) {
        sgemm_load_a<MT, TA, TRI>(A, lda, M, m0, k_begin, k_end, veca, ra, tid);
        sgemm_load_b<TB, TRI>(B, ldb, N, n0, k_begin, k_end, vecb, rb, tid);
        sgemm_store_a<MT, TA>(As[0], ra, tid);
        sgemm_store_b<TB>(Bs[0], rb, tid);
    }
    __syncthreads();
    int it = 0;
    for (int k0 = k_begin; k0 < k_end; k0 += kSBK, ++it) {
        const int cur = it & 1;
        const bool more = k0 + kSBK < k_end;
        if (more) {
            sgemm_load_a<MT, TA, TRI>(A, lda, M, m0, k0 + kSBK, k_end, veca, ra, tid);
            sgemm_load_b<TB, TRI>(B, ldb, N, n0, k0 + kSBK, k_end, vecb, rb, tid);
        }
#pragma unroll
        for (int kk = 0; kk < kSBK; ++kk) {
            float a[4 * MT], b[8];
            const float4 a0 = *reinterpret_cast<const float4*>(&As[cur][kk][tm * 4]);
            a[0] = a0.x; a[1] = a0.y; a[2] = a0.z; a[3] = a0.w;
            if (MT == 2) {
                const float4 a1 = *reinterpret_cast<const float4*>(&As[cur][kk][64 + tm * 4]);
                a[4 * MT - 4] = a1.x; a[4 * MT - 3] = a1.y; a[4 * MT - 2] = a1.z; a[4 * MT - 1] = a1.w;
            }
            const float4 b0 = *reinterpret_cast<const float4*>(&Bs[cur][kk][tn * 4]);
            const float4 b1 = *reinterpret_cast<const float4*>(&Bs[cur][kk][64 + tn * 4]);
            b[0] = b0.x; b[1] = b0.y; b[2] = b0.z; b[3] = b0.w;
            b[4] = b1.x; b[5] = b1.y; b[6] = b1.z; b[7] = b1.w;
#pragma unroll
            for (int i = 0; i < 4 * MT; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        if (more) {
            sgemm_store_a<MT, TA>(As[cur ^ 1], ra, tid);
            sgemm_store_b<TB>(Bs[cur ^ 1], rb, tid);
        }
        __syncthreads();
    }
    // epilogue: rows tm*4 + [0,4) (+64), columns tn*4 + [0,4) and 64 + tn*4 + [0,4)
    const bool vecc = ((reinterpret_cast<uintptr_t>(C) & 15) == 0) && (ldc & 3) == 0;
    const bool vecp = (M & 3) == 0;
#pragma unroll
    for (int h = 0; h < MT; ++h) {
        const int gm = m0 + h * 64 + tm * 4;
        if (gm >= M) continue;
        const bool full = gm + 3 < M;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int gn = n0 + (j < 4 ? tn * 4 + j : 64 + tn * 4 + j - 4);
            if (gn >= N) continue;
            float o[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) o[r] = acc[h * 4 + r][j];
            if (partial) {
                float* p = partial + (int64_t)blockIdx.z * M * N + gm + (int64_t)gn * M;
                if (full && vecp) {
                    *reinterpret_cast<float4*>(p) = make_float4(o[0], o[1], o[2], o[3]);
                } else {
#pragma unroll
                    for (int r = 0; r < 4; ++r)
                        if (gm + r < M) p[r] = o[r];
                }
            } else {
                float* c = C + gm + (int64_t)gn * ldc;
                if (full && vecc) {
                    float4 cv = make_float4(alpha * o[0], alpha * o[1], alpha * o[2], alpha * o[3]);
                    if (beta != 0.f) {
                        const float4 old = *reinterpret_cast<const float4*>(c);
                        cv.x = fmaf(beta, old.x, cv.x);
                        cv.y = fmaf(beta, old.y, cv.y);
                        cv.z = fmaf(beta, old.z, cv.z);
                        cv.w = fmaf(beta, old.w, cv.w);
                    }
                    *reinterpret_cast<float4*>(c) = cv;
                } else {
#pragma unroll
                    for (int r = 0; r < 4; ++r) {
                        if (gm + r >= M) continue;
                        float v = alpha * o[r];
                        if (beta != 0.f) v = fmaf(beta, c[r], v);
                        c[r] = v;
                    }
                }
            }
        }
    }
}

// Small outputs from many splits: one warp per output element, lanes over
// the splits (strided), a fixed shuffle tree combining the lanes.
template <typename T>
__global__ void __launch_bounds__(256)
k_splitk_reduce_warp(int M, int N, int splits, T alpha, const T* __restrict__ partial, T beta,
                     T* __restrict__ C, int64_t ldc)
{
    pdl_wait();
    const int64_t total = (int64_t)M * N;
    const int lane = threadIdx.x & 31;
    const int64_t e = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    if (e >= total) return;
    T s = T(0);
    for (int z = lane; z < splits; z += 32) s += partial[(int64_t)z * total + e];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
        T* c = C + (int)(e % M) + (e / M) * ldc;
        T v = alpha * s;
        if (beta != T(0)) v += beta * *c;
        *c = v;
    }
}

template <typename T>
__global__ void k_splitk_reduce(int M, int N, int splits, T alpha, const T* __restrict__ partial,
                                T beta, T* __restrict__ C, int64_t ldc)
{
    pdl_wait();
    int64_t total = (int64_t)M * N;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        // splits summed in order, eight loads in flight (up to 128 splits of a
        // small output: a load-add chain would wait on L2 once per split)
        T s = T(0);
        int z = 0;
        for (; z + 8 <= splits; z += 8) {
            T v[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) v[q] = partial[(int64_t)(z + q) * total + e];
#pragma unroll
            for (int q = 0; q < 8; ++q) s += v[q];
        }
        for (; z < splits; ++z) s += partial[(int64_t)z * total + e];
        int gm = (int)(e % M);
        int64_t gn = e / M;
        T* c = C + gm + gn * ldc;
        T v = alpha * s;
        if (beta != T(0)) v += beta * *c;
        *c = v;
    }
}

template <typename T>
inline void splitk_reduce_launch(int M, int N, int splits, T alpha, const T* partial, T beta, T* C,
                                 int64_t ldc, cudaStream_t st)
{
    const int64_t total = (int64_t)M * N;
    if (splits >= 16 && total <= 65536) {
        const unsigned g = (unsigned)((total * 32 + 255) / 256);
        launch_k(k_splitk_reduce_warp<T>, g, 256, 0, st, M, N, splits, alpha, partial, beta, C, ldc);
    } else {
        unsigned g = (unsigned)((total + 255) / 256);
        if (g > 152 * 8) g = 152 * 8;
        launch_k(k_splitk_reduce<T>, g, 256, 0, st, M, N, splits, alpha, partial, beta, C, ldc);
    }
    SKL_LAUNCHED();
}

// Picks a split-K factor so that the grid covers the GPU when the output is
// small and K is long (down to 64 rows of K per split, up to 128 splits: a
// 64 x 64 Gram over 8,000 rows then runs on 64 CTAs instead of 16).  partial
// must hold splits*M*N entries when splits > 1.
constexpr int kSplitMinK = 64;
constexpr int kSplitMax = 128;
inline int gemm_splits(int M, int N, int K)
{
    int tiles = ((M + kGBM - 1) / kGBM) * ((N + kGBN - 1) / kGBN);
    int s = 1;
    while (tiles * s < 2 * 152 && K / (s * 2) >= kSplitMinK && s < kSplitMax) s *= 2;
    return s;
}

template <int MT, int TRI>
inline void launch_sgemm(bool ta, bool tb, dim3 grid, cudaStream_t st, int M, int N, int K, float alpha,
                         const float* A, int64_t lda, const float* B, int64_t ldb, float beta, float* C,
                         int64_t ldc, int kchunk, float* part)
{
    if (!ta && !tb) launch_k(k_sgemm<MT, false, false, TRI>, grid, 256, 0, st, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, kchunk, part);
    else if (ta && !tb) launch_k(k_sgemm<MT, true, false, TRI>, grid, 256, 0, st, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, kchunk, part);
    else if (!ta && tb) launch_k(k_sgemm<MT, false, true, TRI>, grid, 256, 0, st, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, kchunk, part);
    else launch_k(k_sgemm<MT, true, true, TRI>, grid, 256, 0, st, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, kchunk, part);
}

// Split-K factor for the FP32 kernel (tile bm x 128): fill about two waves.
// A triangular operand leaves half the tile-K work, so it counts half the tiles.
inline int sgemm_splits(int M, int N, int K, int bm, int tri)
{
    int tiles = ((M + bm - 1) / bm) * ((N + kSBN - 1) / kSBN);
    if (tri) tiles = (tiles + 1) / 2;
    int s = 1;
    while (tiles * s < 2 * 152 && K / (s * 2) >= kSplitMinK && s < kSplitMax) s *= 2;
    return s;
}

template <typename T>
inline void gemm_launch_generic(bool ta, bool tb, int M, int N, int K, T alpha, const T* A,
                                int64_t lda, const T* B, int64_t ldb, T beta, T* C, int64_t ldc,
                                T* partial, int64_t partial_cap, int tri, cudaStream_t st)
{
    if (M <= 0 || N <= 0) return;
    int splits = (K > 0 && partial && tri == 0) ? gemm_splits(M, N, K) : 1;
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
    if (tri == 1) launch_k(k_gemm<T, false, false, 1>, grid, 256, 0, st, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, kchunk, part,
                                  (int64_t)0, (int64_t)0, (int64_t)0);
    else if (tri == 2) launch_k(k_gemm<T, false, false, 2>, grid, 256, 0, st, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, kchunk, part,
                                  (int64_t)0, (int64_t)0, (int64_t)0);
    else if (!ta && !tb) launch_k(k_gemm<T, false, false>, grid, 256, 0, st, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, kchunk, part,
                                  (int64_t)0, (int64_t)0, (int64_t)0);
    else if (ta && !tb) launch_k(k_gemm<T, true, false>, grid, 256, 0, st, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, kchunk, part,
                                  (int64_t)0, (int64_t)0, (int64_t)0);
    else if (!ta && tb) launch_k(k_gemm<T, false, true>, grid, 256, 0, st, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, kchunk, part,
                                  (int64_t)0, (int64_t)0, (int64_t)0);
    else launch_k(k_gemm<T, true, true>, grid, 256, 0, st, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, kchunk, part,
                                  (int64_t)0, (int64_t)0, (int64_t)0);
    SKL_LAUNCHED();
    if (splits > 1) {
        splitk_reduce_launch<T>(M, N, splits, alpha, partial, beta, C, ldc, st);
    }
}

template <typename T>
inline void gemm_launch(bool ta, bool tb, int M, int N, int K, T alpha, const T* A, int64_t lda,
                        const T* B, int64_t ldb, T beta, T* C, int64_t ldc, T* partial,
                        int64_t partial_cap, int tri, cudaStream_t st)
{
    gemm_launch_generic<T>(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, partial,
                           partial_cap, tri, st);
}

template <>
inline void gemm_launch<float>(bool ta, bool tb, int M, int N, int K, float alpha, const float* A,
                               int64_t lda, const float* B, int64_t ldb, float beta, float* C,
                               int64_t ldc, float* partial, int64_t partial_cap, int tri,
                               cudaStream_t st)
{
    if (M <= 0 || N <= 0) return;
    const int bm = M <= 64 ? 64 : 128;
    {
        // small outputs with a short K: the 64 x 64 kernel spreads them over
        // more CTAs than the 128-wide tiles would
        const int64_t tiles = (int64_t)((M + bm - 1) / bm) * ((N + kSBN - 1) / kSBN);
        const bool can_split = K > 0 && partial && K >= 512;
        if (!can_split && tiles < 152) {
            gemm_launch_generic<float>(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, partial,
                                       partial_cap, tri, st);
            return;
        }
    }
    // triangular operands split K too: a split's range is intersected with the
    // triangle's per tile (an empty intersection writes a zero partial)
    int splits = (K > 0 && partial) ? sgemm_splits(M, N, K, bm, tri) : 1;
    while (splits > 1 && (int64_t)splits * M * N > partial_cap) splits >>= 1;
    int kchunk = K;
    if (splits > 1) {
        kchunk = (K + splits - 1) / splits;
        kchunk = (kchunk + kSBK - 1) / kSBK * kSBK;
        splits = (K + kchunk - 1) / kchunk;
    }
    if (K <= 0) { kchunk = 0; splits = 1; }
    dim3 grid((M + bm - 1) / bm, (N + kSBN - 1) / kSBN, splits);
    float* part = splits > 1 ? partial : nullptr;
    if (bm == 64) {
        if (tri == 1) launch_sgemm<1, 1>(false, false, grid, st, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, kchunk, part);
        else if (tri == 2) launch_sgemm<1, 2>(false, false, grid, st, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, kchunk, part);
        else launch_sgemm<1, 0>(ta, tb, grid, st, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, kchunk, part);
    } else {
        if (tri == 1) launch_sgemm<2, 1>(false, false, grid, st, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, kchunk, part);
        else if (tri == 2) launch_sgemm<2, 2>(false, false, grid, st, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, kchunk, part);
        else launch_sgemm<2, 0>(ta, tb, grid, st, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, kchunk, part);
    }
    SKL_LAUNCHED();
    if (splits > 1) {
        splitk_reduce_launch<float>(M, N, splits, alpha, partial, beta, C, ldc, st);
    }
}

template <typename T>
void gemm(bool ta, bool tb, int M, int N, int K, T alpha, const T* A, int64_t lda, const T* B,
          int64_t ldb, T beta, T* C, int64_t ldc, T* partial, int64_t partial_cap,
          cudaStream_t st)
{
    gemm_launch<T>(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, partial, partial_cap, 0, st);
}

// C = alpha * A * B + beta * C with A upper triangular (tri = 1) or B upper
// triangular (tri = 2); no transposes; split-K (FP32) when a partial buffer
// is given.
template <typename T>
void trmm(int tri, int M, int N, int K, T alpha, const T* A, int64_t lda, const T* B, int64_t ldb,
          T beta, T* C, int64_t ldc, cudaStream_t st, T* partial = nullptr, int64_t partial_cap = 0)
{
    gemm_launch<T>(false, false, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, partial, partial_cap, tri,
                   st);
}

// batch products C_z = alpha op(A_z) op(B_z) + beta C_z, z = 0..batch-1, with
// A_z = A + z bsa etc. (one launch; tri as in trmm)
template <typename T>
void trmm_batched(int tri, int M, int N, int K, T alpha, const T* A, int64_t lda, int64_t bsa,
                  const T* B, int64_t ldb, int64_t bsb, T beta, T* C, int64_t ldc, int64_t bsc,
                  int batch, cudaStream_t st)
{
    if (M <= 0 || N <= 0 || batch <= 0) return;
    dim3 grid((M + kGBM - 1) / kGBM, (N + kGBN - 1) / kGBN, batch);
    if (tri == 1)
        launch_k(k_gemm<T, false, false, 1, true>, grid, 256, 0, st, M, N, K, alpha, A, lda, B, ldb, beta, C,
                                                                ldc, K, nullptr, bsa, bsb, bsc);
    else if (tri == 2)
        launch_k(k_gemm<T, false, false, 2, true>, grid, 256, 0, st, M, N, K, alpha, A, lda, B, ldb, beta, C,
                                                                ldc, K, nullptr, bsa, bsb, bsc);
    else
        launch_k(k_gemm<T, false, false, 0, true>, grid, 256, 0, st, M, N, K, alpha, A, lda, B, ldb, beta, C,
                                                                ldc, K, nullptr, bsa, bsb, bsc);
    SKL_LAUNCHED();
}

}  // namespace skl
