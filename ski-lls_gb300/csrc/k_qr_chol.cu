// k_qr_chol.cu -- the CholeskyQR2 panel of the randomized QR (FP32): the
// tall products as GEMMs over the whole GPU and the b x b algebra
// (Cholesky, triangular inverses, modified LU) in single-CTA kernels.  The
// algorithm and its failure rule are described with the panel loop in
// k_qr.cu.
#include <cmath>
#include <cstdint>
#include <type_traits>

#include "skl_internal.hpp"
#include "launch.cuh"
#include "common.cuh"
#include "k_gemm.cuh"

namespace skl {

constexpr int kSmallThreads = 1024;

// ---- small dense algebra on b x b (b <= 64) row-major shared-memory blocks --
// The factorizations are blocked by 16: the 16 x 16 diagonal blocks are
// factored and inverted by one warp (a step is a __syncwarp, not a block
// barrier), and everything else is a block product over the whole CTA
// (blk_mul).  A 64 x 64 Cholesky plus inverse is then 4 warp factorizations
// and ~14 block barriers instead of 128 one-barrier elimination steps, each of
// which had to wait for all 32 warps of the CTA.  Matrices are padded to
// np = round_up(b, 16) rows/columns (identity for the Cholesky, zeros for the
// LU input, which the modified LU turns into identity factors).
constexpr int kDB = 16;   // diagonal block

// Warp-level 16 x 16 routines: lane l holds row l >> 1, columns 8 (l & 1) ..
// +7 of the block in registers; row k reaches the other lanes by shuffles, so
// a step is ~25 instructions with no shared-memory round trip.  The step
// loops stay rolled (register elements picked by selects): a one-warp
// straight-line version would wait on instruction fetch.
template <typename T>
SKL_DEV T sel8(const T (&a)[8], int i)
{
    T v = a[0];
#pragma unroll
    for (int e = 1; e < 8; ++e) v = (i == e) ? a[e] : v;
    return v;
}

// Element k of the lane's own row (k in either half of the row).
template <typename T>
SKL_DEV T own_col(const T (&a)[8], int k, int lane)
{
    const T mine = sel8(a, k & 7);
    const T other = __shfl_xor_sync(0xffffffffu, mine, 1);
    return ((k >> 3) == (lane & 1)) ? mine : other;
}

template <typename T>
SKL_DEV void row_load(const T* A, int ld, T (&a)[8])
{
    const int lane = threadIdx.x & 31, r = lane >> 1, cb = (lane & 1) * 8;
#pragma unroll
    for (int e = 0; e < 8; ++e) a[e] = A[r * ld + cb + e];
}

// In-place Cholesky of the symmetric 16 x 16 block A (both triangles hold the
// current values): R (upper, normalised, zeros below) over A.  Rows stay
// unnormalised during the elimination and are scaled by 1/sqrt(d) at the end.
// Sets *bad when a pivot is not above 32 eps times its mass.
template <typename T>
SKL_DEV T t_rcp(T x);
template <> SKL_DEV float t_rcp<float>(float x) { return __frcp_rn(x); }
template <> SKL_DEV double t_rcp<double>(double x) { return __drcp_rn(x); }

// Pivot reciprocal on the elimination's dependency chain: the hardware
// approximation (relative error ~2^-23, like one more rounding of the
// pivot) instead of the correctly rounded multi-instruction sequence.
template <typename T>
SKL_DEV T t_rcp_chain(T x);
template <> SKL_DEV float t_rcp_chain<float>(float x)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
template <> SKL_DEV double t_rcp_chain<double>(double x) { return __drcp_rn(x); }

// Step k = 8 kh + kl: kl is a compile-time index (the inner loop is unrolled
// by 8) so the pivot and the lane's own column k come from fixed registers.
template <typename T>
SKL_DEV void warp16_chol(T* A, int ld, const T* __restrict__ mass, T eps, int* bad)
{
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, r = lane >> 1, cb = (lane & 1) * 8;
    T a[8];
    row_load(A, ld, a);
    bool isbad = false;
#pragma unroll 1
    for (int kh = 0; kh < 2; ++kh) {
#pragma unroll
        for (int kl = 0; kl < 8; ++kl) {
            const int k = kh * 8 + kl;
            const T d = __shfl_sync(full, a[kl], 2 * k + kh);
            const T ms = mass[k];
            const bool ok = d > T(32) * eps * ms && ms > T(0);
            isbad = isbad || !ok;
            const T inv = ok ? t_rcp_chain(d) : T(0);
            T rk[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) rk[e] = __shfl_sync(full, a[e], 2 * k + (lane & 1));
            const T other = __shfl_xor_sync(full, a[kl], 1);
            const T g = (kh == (lane & 1) ? a[kl] : other) * inv;   // A[r][k] = A[k][r]
            if (r > k) {
#pragma unroll
                for (int e = 0; e < 8; ++e)
                    if (cb + e > k) a[e] -= g * rk[e];
            }
        }
    }
    if (isbad && lane == 0) *bad = 1;
    const T d = own_col(a, r, lane);
    const T sc = d > T(0) ? t_rcp(t_sqrt(d)) : T(0);
#pragma unroll
    for (int e = 0; e < 8; ++e) A[r * ld + cb + e] = (cb + e >= r) ? a[e] * sc : T(0);
    __syncwarp();
}

// X = U^{-1} for the upper 16 x 16 block U (entries below its diagonal never
// read): X's upper triangle, and zeros below it when zero_lower.
template <typename T>
SKL_DEV void warp16_inv_upper(const T* U, int ldu, T* X, int ldx, bool zero_lower)
{
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, r = lane >> 1, cb = (lane & 1) * 8;
    const T iv = lane < kDB ? t_rcp(U[lane * ldu + lane]) : T(0);
    T x[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) x[e] = (cb + e == r) ? T(1) : T(0);
#pragma unroll 1
    for (int k = kDB - 1; k >= 0; --k) {
        const T ik = __shfl_sync(full, iv, k);
        const T u = U[r * ldu + k];
        if (r == k) {
#pragma unroll
            for (int e = 0; e < 8; ++e) x[e] *= ik;
        }
        T xk[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) xk[e] = __shfl_sync(full, x[e], 2 * k + (lane & 1));
        if (r < k) {
#pragma unroll
            for (int e = 0; e < 8; ++e) x[e] -= u * xk[e];
        }
    }
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        const int c = cb + e;
        if (c >= r) X[r * ldx + c] = x[e];
        else if (zero_lower) X[r * ldx + c] = T(0);
    }
    __syncwarp();
}

// Y = L^{-1} for the unit lower 16 x 16 block L (strict lower part read):
// Y's strict lower part only (unit diagonal implied).
template <typename T>
SKL_DEV void warp16_inv_unit_lower(const T* L, int ldl, T* Y, int ldy)
{
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, r = lane >> 1, cb = (lane & 1) * 8;
    T y[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) y[e] = T(0);
#pragma unroll 1
    for (int k = 0; k < kDB - 1; ++k) {
        const T l = L[r * ldl + k];
        T yk[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) yk[e] = __shfl_sync(full, y[e], 2 * k + (lane & 1));
        if (r > k) {
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                const int c = cb + e;
                if (c < k) y[e] -= l * yk[e];
                else if (c == k) y[e] -= l;
            }
        }
    }
#pragma unroll
    for (int e = 0; e < 8; ++e)
        if (cb + e < r) Y[r * ldy + cb + e] = y[e];
    __syncwarp();
}

// Modified LU without pivoting of the 16 x 16 block A in place: S_k =
// -sign(pivot), U_kk = pivot - S_k (|U_kk| >= 1); L's multipliers below the
// diagonal, U on and above; S to sg.
template <typename T>
SKL_DEV void warp16_mlu(T* A, int ld, T* sg)
{
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, r = lane >> 1, cb = (lane & 1) * 8;
    T a[8];
    row_load(A, ld, a);
#pragma unroll 1
    for (int kh = 0; kh < 2; ++kh) {
#pragma unroll
        for (int kl = 0; kl < 8; ++kl) {
            const int k = kh * 8 + kl;
            const T p = __shfl_sync(full, a[kl], 2 * k + kh);
            const T sk = p >= T(0) ? T(-1) : T(1);
            const T ukk = p - sk;
            const T iu = t_rcp_chain(ukk);
            T rk[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) rk[e] = __shfl_sync(full, a[e], 2 * k + (lane & 1));
            const T other = __shfl_xor_sync(full, a[kl], 1);
            const T l = (kh == (lane & 1) ? a[kl] : other) * iu;
            if (r > k) {
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const int c = cb + e;
                    if (c > k) a[e] -= l * rk[e];
                    else if (c == k) a[e] = l;
                }
            } else if (r == k) {
                if (kh == (lane & 1)) a[kl] = ukk;
            }
            if (lane == 0) sg[k] = sk;
        }
    }
#pragma unroll
    for (int e = 0; e < 8; ++e) A[r * ld + cb + e] = a[e];
    __syncwarp();
}

// Operand views for blk_mul, in the coordinates (r, s) of op(X):
enum : int { kMFull = 0, kMUpper = 1, kMUpperUnit = 2, kMLowerUnit = 3 };

template <typename T, bool TR, int MASK>
SKL_DEV T op_at(const T* X, int ld, int r, int s)
{
    if (MASK == kMUpper && s < r) return T(0);
    if (MASK == kMUpperUnit && s <= r) return s == r ? T(1) : T(0);
    if (MASK == kMLowerUnit && s >= r) return s == r ? T(1) : T(0);
    return TR ? X[s * ld + r] : X[r * ld + s];
}

// k range of a product term for masked operands: A upper restricts k >= i,
// B upper / upper-unit restricts k <= c, A lower-unit restricts k <= i.
template <int MA, int MB>
SKL_DEV void k_range(int i0, int c0, int tr, int tc, int kk, int& klo, int& khi)
{
    klo = 0;
    khi = kk;
    if (MA == kMUpper) klo = i0;
    if (MA == kMLowerUnit) khi = min(khi, i0 + tr);
    if (MB == kMUpper || MB == kMUpperUnit) khi = min(khi, c0 + tc);
    if (MB == kMLowerUnit) klo = max(klo, c0);
}

// C (m x n) = alpha * op(A) (m x kk) * op(B) (kk x n) [* diag(sB) on B's
// rows] (+ C when ACC), row-major shared memory; TR x TR register tiles, one
// per thread (m * n <= TR * TR * kSmallThreads); k runs only over the range
// the operand masks leave nonzero.  Results wait for a block barrier, so C may
// alias A or B.  With Cg set, C goes to global memory column-major (ldg)
// instead and its diagonal also to tau.
template <typename T, bool TA, int MA, bool TB, int MB, bool ACC, int TR>
SKL_DEV void blk_mul_t(int m, int n, int kk, const T* A, int lda, const T* B, int ldb,
                       const T* __restrict__ sB, T alpha, T* C, int ldc, T* __restrict__ Cg, int ldg,
                       T* __restrict__ tau)
{
    const int ntc = (n + TR - 1) / TR;
    const int t = threadIdx.x;
    const int i0 = (t / ntc) * TR, c0 = (t % ntc) * TR;
    const bool act = i0 < m;
    T acc[TR][TR];
#pragma unroll
    for (int r = 0; r < TR; ++r)
#pragma unroll
        for (int q = 0; q < TR; ++q) acc[r][q] = T(0);
    if (act) {
        int klo, khi;
        k_range<MA, MB>(i0, c0, TR, TR, kk, klo, khi);
#pragma unroll 4
        for (int k = klo; k < khi; ++k) {
            T av[TR], bv[TR];
#pragma unroll
            for (int r = 0; r < TR; ++r) av[r] = (i0 + r < m) ? op_at<T, TA, MA>(A, lda, i0 + r, k) : T(0);
            const T sc = sB ? sB[k] : T(1);
#pragma unroll
            for (int q = 0; q < TR; ++q) bv[q] = (c0 + q < n) ? sc * op_at<T, TB, MB>(B, ldb, k, c0 + q) : T(0);
#pragma unroll
            for (int r = 0; r < TR; ++r)
#pragma unroll
                for (int q = 0; q < TR; ++q) acc[r][q] += av[r] * bv[q];
        }
    }
    __syncthreads();
    if (act) {
#pragma unroll
        for (int r = 0; r < TR; ++r) {
            const int i = i0 + r;
            if (i >= m) continue;
#pragma unroll
            for (int q = 0; q < TR; ++q) {
                const int c = c0 + q;
                if (c >= n) continue;
                const T v = alpha * acc[r][q];
                if (Cg) {
                    Cg[i + (int64_t)c * ldg] = v;
                    if (i == c) tau[i] = v;
                } else if (ACC) {
                    C[i * ldc + c] += v;
                } else {
                    C[i * ldc + c] = v;
                }
            }
        }
    }
    __syncthreads();
}

// FP32: the same product on the warps' tensor cores, one 16 x 8 tile of C per
// warp (mma.sync m16n8k8 TF32; a 64 x 64 result is the CTA's 32 warps), k
// over the range the masks leave nonzero.  3xTF32 with round-to-nearest
// splits, hi = rna(a) and lo = rna(a - hi), so hi*hi + hi*lo + lo*hi carries
// each product to ~2^-24 like an FP32 FMA.  A 64 x 64 x 64 product is ~200
// instructions per warp instead of ~770 per thread for the 2 x 2 register
// tiles, and these products are most of the panel's serial b x b algebra.
// (For a single-CTA product this small the warp-level MMA beats a tcgen05
// launch: no tensor-memory allocation, descriptors or commit round trip.)
SKL_DEV unsigned tf32_rna(float a)
{
    unsigned r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(a));
    return r;
}

SKL_DEV void mma_tf32_16x8x8(float (&d)[4], const unsigned (&a)[4], const unsigned (&b)[2])
{
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, "
        "{%8, %9}, {%0, %1, %2, %3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// One warp's 16 x 8 tile w of C = op(A) op(B) (m x n, k over the masks'
// range), accumulated in acc; false when the product has no tile w.
template <bool TA, int MA, bool TB, int MB>
SKL_DEV bool tc_tile(int w, int m, int n, int kk, const float* A, int lda, const float* B, int ldb,
                     const float* __restrict__ sB, float (&acc)[4], int& i0, int& c0)
{
    const int lane = threadIdx.x & 31;
    const int g = lane >> 2, tig = lane & 3;
    const int ntn = (n + 7) >> 3;
    acc[0] = acc[1] = acc[2] = acc[3] = 0.f;
    if (w < 0 || w >= ((m + 15) >> 4) * ntn) return false;
    i0 = (w / ntn) * 16;
    c0 = (w % ntn) * 8;
    int klo, khi;
    k_range<MA, MB>(i0, c0, 16, 8, kk, klo, khi);
    klo &= ~7;
    const int ra0 = i0 + g, ra1 = i0 + g + 8, cb = c0 + g;
    for (int k0 = klo; k0 < khi; k0 += 8) {
        const int ka0 = k0 + tig, ka1 = k0 + tig + 4;
        // fragments: A (g, tig) (g+8, tig) (g, tig+4) (g+8, tig+4); B (tig, g) (tig+4, g)
        float av[4], bv[2];
        av[0] = (ra0 < m && ka0 < kk) ? op_at<float, TA, MA>(A, lda, ra0, ka0) : 0.f;
        av[1] = (ra1 < m && ka0 < kk) ? op_at<float, TA, MA>(A, lda, ra1, ka0) : 0.f;
        av[2] = (ra0 < m && ka1 < kk) ? op_at<float, TA, MA>(A, lda, ra0, ka1) : 0.f;
        av[3] = (ra1 < m && ka1 < kk) ? op_at<float, TA, MA>(A, lda, ra1, ka1) : 0.f;
        bv[0] = (ka0 < kk && cb < n) ? (sB ? sB[ka0] : 1.f) * op_at<float, TB, MB>(B, ldb, ka0, cb) : 0.f;
        bv[1] = (ka1 < kk && cb < n) ? (sB ? sB[ka1] : 1.f) * op_at<float, TB, MB>(B, ldb, ka1, cb) : 0.f;
        unsigned ah[4], al[4], bh[2], bl[2];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            ah[e] = tf32_rna(av[e]);
            al[e] = tf32_rna(av[e] - __uint_as_float(ah[e]));
        }
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            bh[e] = tf32_rna(bv[e]);
            bl[e] = tf32_rna(bv[e] - __uint_as_float(bh[e]));
        }
        mma_tf32_16x8x8(acc, al, bh);
        mma_tf32_16x8x8(acc, ah, bl);
        mma_tf32_16x8x8(acc, ah, bh);
    }
    return true;
}

// C fragment: (g, 2 tig) (g, 2 tig + 1) (g + 8, 2 tig) (g + 8, 2 tig + 1)
template <bool ACC>
SKL_DEV void tc_tile_store(int m, int n, int i0, int c0, const float (&acc)[4], float alpha, float* C, int ldc,
                           float* __restrict__ Cg, int ldg, float* __restrict__ tau)
{
    const int lane = threadIdx.x & 31;
    const int g = lane >> 2, tig = lane & 3;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const int i = i0 + g + (e >> 1) * 8, c = c0 + 2 * tig + (e & 1);
        if (i >= m || c >= n) continue;
        const float v = alpha * acc[e];
        if (Cg) {
            Cg[i + (int64_t)c * ldg] = v;
            if (i == c) tau[i] = v;
        } else if (ACC) {
            C[i * ldc + c] += v;
        } else {
            C[i * ldc + c] = v;
        }
    }
}

template <bool TA, int MA, bool TB, int MB, bool ACC>
SKL_DEV void blk_mul_tc(int m, int n, int kk, const float* A, int lda, const float* B, int ldb,
                        const float* __restrict__ sB, float alpha, float* C, int ldc,
                        float* __restrict__ Cg, int ldg, float* __restrict__ tau)
{
    float acc[4];
    int i0 = 0, c0 = 0;
    const bool act = tc_tile<TA, MA, TB, MB>(threadIdx.x >> 5, m, n, kk, A, lda, B, ldb, sB, acc, i0, c0);
    __syncthreads();
    if (act) tc_tile_store<ACC>(m, n, i0, c0, acc, alpha, C, ldc, Cg, ldg, tau);
    __syncthreads();
}

// Tiles of a product: the warps a phase gives it.
SKL_DEV int tc_tiles(int m, int n) { return ((m + 15) >> 4) * ((n + 7) >> 3); }

// Off-diagonal blocks of X = U^{-1} (upper) and, when L is given, of Y =
// L^{-1} (unit lower), np x np (np a multiple of 16, at most 64), once the
// 16 x 16 diagonal blocks hold the inverses: recursive doubling,
//   [A B; 0 C]^{-1} = [A^{-1}, -A^{-1} B C^{-1}; 0, C^{-1}],
//   [A 0; B C]^{-1} = [A^{-1}, 0; -C^{-1} B A^{-1}, C^{-1}],
// with every pair of a level (and the U and L pairs) in one phase of warp
// tiles: two block barriers per product level instead of two per product.
// tmp holds 64 x 36 (ldt = 36): U pairs in rows 0..31, L pairs in 32..63,
// pair q of a level at column 16 q.
SKL_DEV void inv_offdiag_tc(const float* U, int ldu, float* X, int ldx, const float* L, int ldl, float* Y,
                            int ldy, int np, float* tmp, int ldt)
{
    const int warp = threadIdx.x >> 5;
    for (int w = kDB; w < np; w *= 2) {
        // phase 1: tmp_U = U_12 X_22, tmp_L = L_21 Y_11 for every pair
        {
            float acc[4];
            int i0 = 0, c0 = 0, m = 0, n = 0;
            float* C = nullptr;
            bool act = false;
            int base = 0;
            for (int p0 = 0; p0 + w < np; p0 += 2 * w) {
                const int n2 = min(w, np - p0 - w), q = p0 / (2 * w);
                const int tU = tc_tiles(w, n2);
                if (warp >= base && warp < base + tU) {
                    act = tc_tile<false, kMFull, false, kMUpper>(warp - base, w, n2, n2, U + p0 * ldu + p0 + w,
                                                                 ldu, X + (p0 + w) * ldx + p0 + w, ldx,
                                                                 nullptr, acc, i0, c0);
                    C = tmp + 16 * q;
                    m = w;
                    n = n2;
                }
                base += tU;
                if (L) {
                    const int tL = tc_tiles(n2, w);
                    if (warp >= base && warp < base + tL) {
                        act = tc_tile<false, kMFull, false, kMLowerUnit>(warp - base, n2, w, w,
                                                                         L + (p0 + w) * ldl + p0, ldl,
                                                                         Y + p0 * ldy + p0, ldy, nullptr, acc,
                                                                         i0, c0);
                        C = tmp + 32 * ldt + 16 * q;
                        m = n2;
                        n = w;
                    }
                    base += tL;
                }
            }
            __syncthreads();
            if (act) tc_tile_store<false>(m, n, i0, c0, acc, 1.f, C, ldt, nullptr, 0, nullptr);
            __syncthreads();
        }
        // phase 2: X_12 = -X_11 tmp_U, Y_21 = -Y_22 tmp_L
        {
            float acc[4];
            int i0 = 0, c0 = 0, m = 0, n = 0, ldc = 0;
            float* C = nullptr;
            bool act = false;
            int base = 0;
            for (int p0 = 0; p0 + w < np; p0 += 2 * w) {
                const int n2 = min(w, np - p0 - w), q = p0 / (2 * w);
                const int tU = tc_tiles(w, n2);
                if (warp >= base && warp < base + tU) {
                    act = tc_tile<false, kMUpper, false, kMFull>(warp - base, w, n2, w, X + p0 * ldx + p0, ldx,
                                                                 tmp + 16 * q, ldt, nullptr, acc, i0, c0);
                    C = X + p0 * ldx + p0 + w;
                    ldc = ldx;
                    m = w;
                    n = n2;
                }
                base += tU;
                if (L) {
                    const int tL = tc_tiles(n2, w);
                    if (warp >= base && warp < base + tL) {
                        act = tc_tile<false, kMLowerUnit, false, kMFull>(warp - base, n2, w, n2,
                                                                         Y + (p0 + w) * ldy + p0 + w, ldy,
                                                                         tmp + 32 * ldt + 16 * q, ldt, nullptr,
                                                                         acc, i0, c0);
                        C = Y + (p0 + w) * ldy + p0;
                        ldc = ldy;
                        m = n2;
                        n = w;
                    }
                    base += tL;
                }
            }
            __syncthreads();
            if (act) tc_tile_store<false>(m, n, i0, c0, acc, -1.f, C, ldc, nullptr, 0, nullptr);
            __syncthreads();
        }
    }
}

// 2 x 2 tiles for FP64: 4 x 4 tiles measured slower inside the small kernels
// (their k ranges trim less under the triangular masks).
template <typename T, bool TA, int MA, bool TB, int MB, bool ACC = false>
SKL_DEV void blk_mul(int m, int n, int kk, const T* A, int lda, const T* B, int ldb,
                     const T* __restrict__ sB, T alpha, T* C, int ldc, T* __restrict__ Cg = nullptr,
                     int ldg = 0, T* __restrict__ tau = nullptr)
{
    if constexpr (std::is_same<T, float>::value)
        blk_mul_tc<TA, MA, TB, MB, ACC>(m, n, kk, A, lda, B, ldb, sB, alpha, C, ldc, Cg, ldg, tau);
    else
        blk_mul_t<T, TA, MA, TB, MB, ACC, 2>(m, n, kk, A, lda, B, ldb, sB, alpha, C, ldc, Cg, ldg, tau);
}

// Off-diagonal blocks of X = U^{-1} (np x np upper, np a multiple of 16)
// once X's 16 x 16 diagonal blocks hold the inverses of U's: recursive
// doubling, [A B; 0 C]^{-1} = [A^{-1}, -A^{-1} B C^{-1}; 0, C^{-1}].  tmp holds
// 32 x 32 (ldt).
template <typename T>
SKL_DEV void inv_upper_offdiag(const T* U, int ldu, T* X, int ldx, int np, T* tmp, int ldt)
{
    for (int w = kDB; w < np; w *= 2) {
        for (int p0 = 0; p0 + w < np; p0 += 2 * w) {
            const int n2 = min(w, np - p0 - w);
            blk_mul<T, false, kMFull, false, kMUpper>(w, n2, n2, U + p0 * ldu + p0 + w, ldu,
                                                     X + (p0 + w) * ldx + p0 + w, ldx, nullptr, T(1),
                                                     tmp, ldt);
            blk_mul<T, false, kMUpper, false, kMFull>(w, n2, w, X + p0 * ldx + p0, ldx, tmp, ldt,
                                                     nullptr, T(-1), X + p0 * ldx + p0 + w, ldx);
        }
    }
}

// Strict lower off-diagonal blocks of Y = L^{-1} (np x np unit lower) once
// Y's diagonal blocks hold the inverses of L's:
// [A 0; B C]^{-1} = [A^{-1}, 0; -C^{-1} B A^{-1}, C^{-1}].
template <typename T>
SKL_DEV void inv_unit_lower_offdiag(const T* L, int ldl, T* Y, int ldy, int np, T* tmp, int ldt)
{
    for (int w = kDB; w < np; w *= 2) {
        for (int p0 = 0; p0 + w < np; p0 += 2 * w) {
            const int n2 = min(w, np - p0 - w);
            blk_mul<T, false, kMFull, false, kMLowerUnit>(n2, w, w, L + (p0 + w) * ldl + p0, ldl,
                                                         Y + p0 * ldy + p0, ldy, nullptr, T(1), tmp,
                                                         ldt);
            blk_mul<T, false, kMLowerUnit, false, kMFull>(n2, w, n2, Y + (p0 + w) * ldy + p0 + w, ldy,
                                                         tmp, ldt, nullptr, T(-1),
                                                         Y + (p0 + w) * ldy + p0, ldy);
        }
    }
}

// Cholesky G = R^T R (np x np, np a multiple of 16) with X = R^{-1}: R (upper,
// zeros below) over G, X (upper, zeros below) to Xs.  Blocked right-looking:
// per 16-block, warp 0 factors the diagonal block and inverts it, then
// R12 = R11^{-T} G12 and G22 -= R12^T R12 as block products.
template <typename T>
SKL_DEV void chol_inv_small(T* G, int ldx, int np, const T* __restrict__ mass, T eps, T* Xs, T* tmp,
                            int ldt, int* bad)
{
    for (int e = threadIdx.x; e < np * np; e += kSmallThreads) Xs[(e / np) * ldx + e % np] = T(0);
    __syncthreads();
    for (int k0 = 0; k0 < np; k0 += kDB) {
        const int rest = np - k0 - kDB;
        T* G11 = G + k0 * ldx + k0;
        if (threadIdx.x < 32) {
            warp16_chol<T>(G11, ldx, mass + k0, eps, bad);
            warp16_inv_upper<T>(G11, ldx, Xs + k0 * ldx + k0, ldx, true);
        }
        __syncthreads();
        if (rest > 0) {
            T* G12 = G11 + kDB;
            blk_mul<T, true, kMFull, false, kMFull>(kDB, rest, kDB, Xs + k0 * ldx + k0, ldx, G12, ldx,
                                                    nullptr, T(1), G12, ldx);
            blk_mul<T, true, kMFull, false, kMFull, true>(rest, rest, kDB, G12, ldx, G12, ldx, nullptr,
                                                          T(-1), G11 + kDB * ldx + kDB, ldx);
        }
    }
    // R's strict lower part (the off-diagonal blocks kept G's values)
    for (int e = threadIdx.x; e < np * np; e += kSmallThreads) {
        const int i = e / np, c = e % np;
        if (c < i) G[i * ldx + c] = T(0);
    }
    __syncthreads();
    if constexpr (std::is_same<T, float>::value)
        inv_offdiag_tc(G, ldx, Xs, ldx, nullptr, 0, nullptr, 0, np, tmp, ldt);
    else
        inv_upper_offdiag<T>(G, ldx, Xs, ldx, np, tmp, ldt);
}

// Modified LU of A (np x np) in place (L strict lower, U upper), signs to
// sg, and in Z: L^{-1} (strict lower, unit diagonal implied) and U^{-1}
// (upper).  Blocked right-looking by 16: warp 0 factors the diagonal block,
// warps 0 and 1 invert its L and U factors into Z, then U12 = L11^{-1} A12,
// L21 = A21 U11^{-1} and A22 -= L21 U12 as block products.
template <typename T>
SKL_DEV void mlu_inv_small(T* A, int ldx, int np, T* sg, T* Z, T* tmp, int ldt)
{
    for (int k0 = 0; k0 < np; k0 += kDB) {
        const int rest = np - k0 - kDB;
        T* A11 = A + k0 * ldx + k0;
        T* Z11 = Z + k0 * ldx + k0;
        if (threadIdx.x < 32) warp16_mlu<T>(A11, ldx, sg + k0);
        __syncthreads();
        if (threadIdx.x < 32) warp16_inv_unit_lower<T>(A11, ldx, Z11, ldx);
        else if (threadIdx.x < 64) warp16_inv_upper<T>(A11, ldx, Z11, ldx, false);
        __syncthreads();
        if (rest > 0) {
            T* A12 = A11 + kDB;
            T* A21 = A11 + kDB * ldx;
            if constexpr (std::is_same<T, float>::value) {
                // U12 = L11^{-1} A12 and L21 = A21 U11^{-1} in one phase
                const int warp = threadIdx.x >> 5, t12 = tc_tiles(kDB, rest);
                float acc[4];
                int i0 = 0, c0 = 0;
                bool act;
                if (warp < t12)
                    act = tc_tile<false, kMLowerUnit, false, kMFull>(warp, kDB, rest, kDB, Z11, ldx, A12, ldx,
                                                                     nullptr, acc, i0, c0);
                else
                    act = tc_tile<false, kMFull, false, kMUpper>(warp - t12, rest, kDB, kDB, A21, ldx, Z11,
                                                                 ldx, nullptr, acc, i0, c0);
                __syncthreads();
                if (act) {
                    if (warp < t12) tc_tile_store<false>(kDB, rest, i0, c0, acc, 1.f, A12, ldx, nullptr, 0, nullptr);
                    else tc_tile_store<false>(rest, kDB, i0, c0, acc, 1.f, A21, ldx, nullptr, 0, nullptr);
                }
                __syncthreads();
            } else {
                blk_mul<T, false, kMLowerUnit, false, kMFull>(kDB, rest, kDB, Z11, ldx, A12, ldx, nullptr,
                                                             T(1), A12, ldx);
                blk_mul<T, false, kMFull, false, kMUpper>(rest, kDB, kDB, A21, ldx, Z11, ldx, nullptr, T(1),
                                                         A21, ldx);
            }
            blk_mul<T, false, kMFull, false, kMFull, true>(rest, rest, kDB, A21, ldx, A12, ldx, nullptr,
                                                           T(-1), A11 + kDB * ldx + kDB, ldx);
        }
    }
    if constexpr (std::is_same<T, float>::value) {
        inv_offdiag_tc(A, ldx, Z, ldx, A, ldx, Z, ldx, np, tmp, ldt);
    } else {
        inv_upper_offdiag<T>(A, ldx, Z, ldx, np, tmp, ldt);
        inv_unit_lower_offdiag<T>(A, ldx, Z, ldx, np, tmp, ldt);
    }
}

// Padded size of the b x b algebra and the workspace layout of the small
// kernels: four np x np blocks (row-major, ld = np + 4), a 64 x 36 product
// scratch, and 3 np entries.
__host__ __device__ inline int small_np(int b) { return (b + kDB - 1) / kDB * kDB; }
template <typename T>
size_t chol_small_smem_bytes(int b)
{
    const size_t np = (size_t)small_np(b);
    return (4 * np * (np + 4) + 64 * 36 + 3 * np) * sizeof(T) + 256;
}

// Pass 1: R1 and X1 = R1^{-1} from G1 (column-major b x b, ldg = b).  Sets
// *fail (1 on a Cholesky breakdown, else 0).
template <typename T>
__global__ void __launch_bounds__(kSmallThreads, 1)
k_chol_small1(const T* __restrict__ G, int b, T* __restrict__ R1, T* __restrict__ X1,
              int* __restrict__ fail)
{
    pdl_wait();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int np = small_np(b);
    const int LDX = np + 4;
    T* S0 = (T*)smem_raw;
    T* S1 = S0 + (size_t)np * LDX;
    T* tmp = S1 + (size_t)np * LDX;
    T* mass = tmp + 64 * 36;
    __shared__ int s_bad;
    const T eps = std::is_same<T, float>::value ? T(5.9604645e-08) : T(1.1102230246251565e-16);
    if (threadIdx.x == 0) s_bad = 0;
    // G padded with the identity beyond b
    for (int e = threadIdx.x; e < np * np; e += kSmallThreads) {
        const int i = e % np, c = e / np;
        S0[i * LDX + c] = (i < b && c < b) ? G[i + c * b] : (i == c ? T(1) : T(0));
    }
    for (int k = threadIdx.x; k < np; k += kSmallThreads) mass[k] = k < b ? G[k * b + k] : T(1);
    __syncthreads();
    chol_inv_small<T>(S0, LDX, np, mass, eps, S1, tmp, 36, &s_bad);
    for (int e = threadIdx.x; e < b * b; e += kSmallThreads) {
        const int i = e / b, c = e % b;
        R1[e] = S0[i * LDX + c];     // row-major b x b
        X1[c * b + i] = S1[i * LDX + c];   // column-major (a GEMM operand)
    }
    if (threadIdx.x == 0) *fail = s_bad ? 1 : 0;
}

// Pass 2 and the reconstruction: from G2 (column-major), R1 (row-major) and
// the first b rows of Q (column-major, ldq) writes W = R2^{-1} U^{-1}
// (column-major b x b), T (ldt), tau, the panel's first b rows of A (R_H on
// and above the diagonal, L below) and of V (unit lower L).  Does nothing if
// pass 1 failed; sets *fail on a pass-2 breakdown (A untouched).
template <typename T>
__global__ void __launch_bounds__(kSmallThreads, 1)
k_chol_small2(const T* __restrict__ G, int b, const T* __restrict__ R1g, const T* __restrict__ Q,
              int64_t ldq, T* __restrict__ A, int64_t ld, int j0, T* __restrict__ V, int64_t ldv,
              T* __restrict__ Tout, int ldt, T* __restrict__ tau_out, T* __restrict__ Wg,
              int* __restrict__ fail)
{
    pdl_wait();
    if (*fail) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int np = small_np(b);
    const int LDX = np + 4;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    T* S0 = (T*)smem_raw;                        // R1 -> R = R2 R1
    T* S1 = S0 + (size_t)np * LDX;               // G2 -> R2 -> L^{-1} \ U^{-1}
    T* S2 = S1 + (size_t)np * LDX;               // X2 -> W
    T* S3 = S2 + (size_t)np * LDX;               // Q(0:b,:) -> Q1 -> L \ U
    T* tmp = S3 + (size_t)np * LDX;              // 64 x 36 product scratch
    T* Sg = tmp + 64 * 36;
    T* mass = Sg + np;
    __shared__ int s_bad;
    const T eps = std::is_same<T, float>::value ? T(5.9604645e-08) : T(1.1102230246251565e-16);
    if (threadIdx.x == 0) s_bad = 0;
    // G2 padded with the identity, Q(0:b,:) with zeros, beyond b
    for (int e = threadIdx.x; e < np * np; e += kSmallThreads) {
        const int i = e % np, c = e / np;
        const bool in = i < b && c < b;
        S1[i * LDX + c] = in ? G[i + c * b] : (i == c ? T(1) : T(0));
        S3[i * LDX + c] = in ? Q[i + (int64_t)c * ldq] : T(0);
        S0[c * LDX + i] = in ? R1g[c * b + i] : (i == c ? T(1) : T(0));   // row-major source
    }
    for (int k = threadIdx.x; k < np; k += kSmallThreads) mass[k] = T(1);
    __syncthreads();
    // Gershgorin distance of G2 from the identity
    for (int i = wid; i < b; i += kSmallThreads / 32) {
        T sabs = T(0);
        for (int c = lane; c < b; c += 32) sabs += t_abs(S1[i * LDX + c] - (c == i ? T(1) : T(0)));
        sabs = warp_sum(sabs);
        if (lane == 0 && !(sabs <= T(0.5))) s_bad = 1;
    }
    __syncthreads();
    if (s_bad) {
        if (threadIdx.x == 0) *fail = 1;
        return;
    }
    chol_inv_small<T>(S1, LDX, np, mass, eps, S2, tmp, 36, &s_bad);  // R2 over S1, X2 -> S2
    if (s_bad) {
        if (threadIdx.x == 0) *fail = 1;
        return;
    }
    blk_mul<T, false, kMFull, false, kMUpper>(b, b, b, S3, LDX, S2, LDX, nullptr, T(1), S3, LDX);   // Q1 = Q(0:b,:) X2
    blk_mul<T, false, kMUpper, false, kMUpper>(b, b, b, S1, LDX, S0, LDX, nullptr, T(1), S0, LDX);  // R = R2 R1
    mlu_inv_small<T>(S3, LDX, np, Sg, S1, tmp, 36);              // Q1 - S = L U; S1 = L^{-1} \ U^{-1}
    blk_mul<T, false, kMUpper, false, kMUpper>(b, b, b, S2, LDX, S1, LDX, nullptr, T(1), S2, LDX);  // W = X2 U^{-1}
    blk_mul<T, false, kMUpper, true, kMUpperUnit>(b, b, b, S3, LDX, S1, LDX, Sg, T(-1), nullptr, 0,
                                                   Tout, ldt, tau_out + j0);   // T = -U S L^{-T}
    for (int e = threadIdx.x; e < b * b; e += kSmallThreads) {
        const int g = e % b, c = e / b;          // column-major targets
        Wg[e] = S2[g * LDX + c];
        const T l = (g > c) ? S3[g * LDX + c] : T(0);
        A[(int64_t)(j0 + g) + (int64_t)(j0 + c) * ld] = (g <= c) ? Sg[g] * S0[g * LDX + c] : l;
        V[(int64_t)g + (int64_t)c * ldv] = (g > c) ? l : (g == c ? T(1) : T(0));
    }
}

// A(j0+b : j0+M, j0 : j0+b) = V(b : M, :) once the panel succeeded.
template <typename T>
__global__ void k_chol_copy_down(const T* __restrict__ V, int64_t ldv, T* __restrict__ A, int64_t ld,
                                 int j0, int M, int b, const int* __restrict__ fail)
{
    pdl_wait();
    if (*fail) return;
    const int rows = M - b;
    const int c = blockIdx.y;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x)
        A[(int64_t)(j0 + b + r) + (int64_t)(j0 + c) * ld] = V[(int64_t)(b + r) + (int64_t)c * ldv];
}

// Host side: one panel P (M x b, column-major, ld) = A(j0:m, j0:j0+b).
template <typename T>
void chol_panel(T* P, int64_t ld, int M, int b, int j0, T* A, T* cg, T* cr1, T* cx1, T* cw, T* tmp,
                T* V, int64_t ldv, T* Tm, int ldt, T* tau, T* part, int64_t part_cap, int* fail,
                cudaStream_t st)
{
    const size_t ssm = chol_small_smem_bytes<T>(b);
    allow_max_dynamic_smem((const void*)k_chol_small1<T>);
    allow_max_dynamic_smem((const void*)k_chol_small2<T>);
    gemm<T>(true, false, b, b, M, T(1), P, ld, P, ld, T(0), cg, b, part, part_cap, st);
    launch_k(k_chol_small1<T>, 1, kSmallThreads, ssm, st, cg, b, cr1, cx1, fail);
    SKL_CUDA(cudaGetLastError());
    SKL_LAUNCHED();
    gemm<T>(false, false, M, b, b, T(1), P, ld, cx1, b, T(0), tmp, M, nullptr, 0, st);
    gemm<T>(true, false, b, b, M, T(1), tmp, M, tmp, M, T(0), cg, b, part, part_cap, st);
    launch_k(k_chol_small2<T>, 1, kSmallThreads, ssm, st, cg, b, cr1, tmp, M, A, ld, j0, V, ldv, Tm, ldt,
                                                    tau, cw, fail);
    SKL_CUDA(cudaGetLastError());
    SKL_LAUNCHED();
    gemm<T>(false, false, M - b, b, b, T(1), tmp + b, M, cw, b, T(0), V + b, ldv, nullptr, 0, st);
    dim3 gc((unsigned)std::max<int64_t>(1, std::min<int64_t>((M - b + 255) / 256, 64)), b);
    launch_k(k_chol_copy_down<T>, gc, 256, 0, st, V, ldv, A, ld, j0, M, b, fail);
    SKL_LAUNCHED();
}

template <>
void chol_panel<double>(double*, int64_t, int, int, int, double*, double*, double*, double*, double*,
                        double*, double*, int64_t, double*, int, double*, double*, int64_t, int*,
                        cudaStream_t)
{
    fail(SKL_ERR_INVALID, "CholeskyQR2 panel: FP32 only");
}

template void chol_panel<float>(float*, int64_t, int, int, int, float*, float*, float*, float*, float*,
                                float*, float*, int64_t, float*, int, float*, float*, int64_t, int*,
                                cudaStream_t);

}  // namespace skl
