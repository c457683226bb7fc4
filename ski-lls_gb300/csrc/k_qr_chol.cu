// k_qr_chol.cu -- the CholeskyQR2 panel of the randomized QR (FP32): the
// tall products as GEMMs over the whole GPU and the b x b algebra
// (Cholesky, triangular inverses, modified LU) in single-CTA kernels.  The
// algorithm and its failure rule are described with the panel loop in
// k_qr.cu.
#include <cmath>
#include <cstdint>
#include <type_traits>

#include "skl_internal.hpp"
#include "common.cuh"
#include "k_gemm.cuh"

namespace skl {

constexpr int kSmallThreads = 1024;
constexpr int kSmallWarps = kSmallThreads / 32;
constexpr int kMaxSmall = 64;

// ---- small dense algebra on b x b (b <= 64) row-major shared-memory blocks --
// Every routine is a rolled loop over elimination steps with one block
// barrier per step; within a step, warps take rows and lanes take columns of
// the block that changes.  (Fully unrolled register versions were tried:
// their straight-line code, executed once, is bound by instruction fetch.)
// The reciprocal of the next pivot is formed by the thread that finishes that
// pivot, one step ahead, so no division sits on the per-step critical path.

// Thread layout of the eliminations: thread t owns row t >> 4 and the four
// columns 4 (t & 15) .. +3 (one float4 of a row; ld = b + 4 keeps rows
// 16-byte aligned), so 1024 threads cover a 64 x 64 block and every step is
// one vector read-modify-write per thread plus one barrier.
template <typename T> struct Quad;
template <> struct Quad<float> { using type = float4; };
template <> struct Quad<double> { using type = double4; };

template <typename T>
SKL_DEV typename Quad<T>::type ld4(const T* p) { return *reinterpret_cast<const typename Quad<T>::type*>(p); }
template <typename T>
SKL_DEV void st4(T* p, typename Quad<T>::type v) { *reinterpret_cast<typename Quad<T>::type*>(p) = v; }
template <typename T, typename V>
SKL_DEV T q_at(const V& v, int e) { return e == 0 ? v.x : e == 1 ? v.y : e == 2 ? v.z : v.w; }
template <typename T, typename V>
SKL_DEV void q_set(V& v, int e, T x)
{
    if (e == 0) v.x = x;
    else if (e == 1) v.y = x;
    else if (e == 2) v.z = x;
    else v.w = x;
}

// In-place Cholesky G = R^T R of the symmetric b x b block G: R (upper,
// zeros below) over G.  Rows stay unnormalised during the elimination and
// are scaled by 1/sqrt(d_i) at the end.  inv: b scratch entries (1/d_k).
// Sets *bad when a pivot is below 32 eps times its mass.
template <typename T>
SKL_DEV void chol_smem(T* G, int ld, int b, const T* __restrict__ mass, T eps, T* inv, int* bad)
{
    const int i = threadIdx.x >> 4, c0 = (threadIdx.x & 15) * 4;
    const bool own = i < b && c0 < b;
    if (threadIdx.x == 0) {
        const T d = G[0];
        const bool ok = d > T(32) * eps * mass[0] && mass[0] > T(0);
        if (!ok) *bad = 1;
        inv[0] = ok ? T(1) / d : T(0);
    }
    __syncthreads();
    for (int k = 0; k < b - 1; ++k) {
        if (own && i > k && c0 + 3 >= i) {
            const T gki = G[k * ld + i] * inv[k];
            auto row = ld4<T>(G + i * ld + c0);
            const auto piv = ld4<T>(G + k * ld + c0);
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int c = c0 + e;
                if (c >= i && c < b) q_set<T>(row, e, q_at<T>(row, e) - gki * q_at<T>(piv, e));
            }
            st4<T>(G + i * ld + c0, row);
            if (i == k + 1 && c0 <= i && i < c0 + 4) {   // next pivot, finished now
                const T v = q_at<T>(row, i - c0);
                const bool ok = v > T(32) * eps * mass[i] && mass[i] > T(0);
                if (!ok) *bad = 1;
                inv[i] = ok ? T(1) / v : T(0);
            }
        }
        __syncthreads();
    }
    if (own) {
        const T s = inv[i] > T(0) ? t_sqrt(inv[i]) : T(0);
        auto row = ld4<T>(G + i * ld + c0);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int c = c0 + e;
            q_set<T>(row, e, (c >= i) ? q_at<T>(row, e) * s : T(0));
        }
        st4<T>(G + i * ld + c0, row);
    }
    __syncthreads();
}

// X = U^{-1} for the upper triangle of the b x b block U (entries below U's
// diagonal never read).  Back substitution over all columns at once: step k
// removes row k's contribution from rows i < k (columns c >= k), and row i
// is final (scaled by 1/U_ii) after step i + 1.  Writes X's upper triangle,
// and zeros below it when zero_lower (otherwise only the upper triangle is
// written, so X may hold another triangle below).  inv: b scratch entries.
template <typename T>
SKL_DEV void inv_upper_smem(const T* U, int ldu, int b, T* X, int ldx, bool zero_lower, T* inv)
{
    const int i = threadIdx.x >> 4, c0 = (threadIdx.x & 15) * 4;
    const bool own = i < b && c0 < b;
    for (int k = threadIdx.x; k < b; k += kSmallThreads) inv[k] = T(1) / U[k * ldu + k];
    __syncthreads();
    if (own) {
        auto row = ld4<T>(X + i * ldx + c0);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int c = c0 + e;
            if (c >= i) q_set<T>(row, e, (c == i) ? (i == b - 1 ? inv[i] : T(1)) : T(0));
            else if (zero_lower) q_set<T>(row, e, T(0));
        }
        st4<T>(X + i * ldx + c0, row);
    }
    __syncthreads();
    for (int k = b - 1; k >= 1; --k) {
        // X[i][c] -= U[i][k] X[k][c] for i < k <= c; row k - 1 is then final
        const bool has_diag = (i == k - 1) && c0 <= i && i < c0 + 4;
        if (own && i < k && (c0 + 3 >= k || has_diag)) {
            const T uik = U[i * ldu + k];
            const T sc = (i == k - 1) ? inv[i] : T(1);
            auto row = ld4<T>(X + i * ldx + c0);
            const auto xk = ld4<T>(X + k * ldx + c0);
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int c = c0 + e;
                if (c >= k && c < b) q_set<T>(row, e, (q_at<T>(row, e) - uik * q_at<T>(xk, e)) * sc);
                else if (c == i && i == k - 1) q_set<T>(row, e, inv[i]);
            }
            st4<T>(X + i * ldx + c0, row);
        }
        __syncthreads();
    }
}

// Y = L^{-1} for the unit lower triangle of L (strict lower part read):
// Y's strict lower part only (unit diagonal implied).  Forward substitution
// over all columns at once: step k removes row k from rows i > k.
template <typename T>
SKL_DEV void inv_unit_lower_smem(const T* L, int ldl, int b, T* Y, int ldy)
{
    const int i = threadIdx.x >> 4, c0 = (threadIdx.x & 15) * 4;
    const bool own = i < b && c0 < b;
    // Y's strict lower part starts at zero; row k of Y is final before step k
    if (own) {
        auto row = ld4<T>(Y + i * ldy + c0);
#pragma unroll
        for (int e = 0; e < 4; ++e)
            if (c0 + e < i) q_set<T>(row, e, T(0));
        st4<T>(Y + i * ldy + c0, row);
    }
    __syncthreads();
    for (int k = 0; k < b - 1; ++k) {
        if (own && i > k && c0 <= k) {
            const T lik = L[i * ldl + k];
            auto row = ld4<T>(Y + i * ldy + c0);
            const auto yk = ld4<T>(Y + k * ldy + c0);
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int c = c0 + e;
                if (c <= k) q_set<T>(row, e, q_at<T>(row, e) - lik * (c == k ? T(1) : q_at<T>(yk, e)));
            }
            st4<T>(Y + i * ldy + c0, row);
        }
        __syncthreads();
    }
}

// Modified LU without pivoting of the b x b block A in place: S_k =
// -sign(pivot), U_kk = pivot - S_k (|U_kk| >= 1); L's multipliers below the
// diagonal, U on and above; S to sg.  iu: b scratch entries (1/U_kk).
// Column k is scaled into multipliers, and U_kk written, one step later, when
// nothing reads them any more.
template <typename T>
SKL_DEV void mlu_smem(T* A, int ld, int b, T* sg, T* iu)
{
    const int i = threadIdx.x >> 4, c0 = (threadIdx.x & 15) * 4;
    const bool own = i < b && c0 < b;
    if (threadIdx.x == 0) {
        const T p = A[0];
        const T sk = p >= T(0) ? T(-1) : T(1);
        sg[0] = sk;
        iu[0] = T(1) / (p - sk);
    }
    __syncthreads();
    for (int k = 0; k < b; ++k) {
        if (own) {
            auto row = ld4<T>(A + i * ld + c0);
            bool dirty = false;
            if (k > 0 && i >= k - 1 && c0 <= k - 1 && k - 1 < c0 + 4) {
                // finish column k - 1: multiplier (i > k-1) or pivot U_{k-1,k-1}
                const int e = k - 1 - c0;
                q_set<T>(row, e, (i == k - 1) ? T(1) / iu[k - 1] : q_at<T>(row, e) * iu[k - 1]);
                dirty = true;
            }
            if (i > k && c0 + 3 > k) {
                const T lik = A[i * ld + k] * iu[k];
                const auto uk = ld4<T>(A + k * ld + c0);
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int c = c0 + e;
                    if (c > k && c < b) q_set<T>(row, e, q_at<T>(row, e) - lik * q_at<T>(uk, e));
                }
                dirty = true;
                if (i == k + 1 && c0 <= i && i < c0 + 4) {   // next pivot, finished now
                    const T v = q_at<T>(row, i - c0);
                    const T sk = v >= T(0) ? T(-1) : T(1);
                    sg[i] = sk;
                    iu[i] = T(1) / (v - sk);
                }
            }
            if (dirty) st4<T>(A + i * ld + c0, row);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) A[(b - 1) * ld + (b - 1)] = T(1) / iu[b - 1];
    __syncthreads();
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
// rows] (+ C when ACC), row-major shared memory; 2 x 2 register tiles, one
// per thread (m * n <= 4 * kSmallThreads); k runs only over the range the
// operand masks leave nonzero.  Results wait for a block barrier, so C may
// alias A or B.  With Cg set, C goes to global memory column-major (ldg)
// instead and its diagonal also to tau.
template <typename T, bool TA, int MA, bool TB, int MB, bool ACC = false>
SKL_DEV void blk_mul(int m, int n, int kk, const T* A, int lda, const T* B, int ldb,
                     const T* __restrict__ sB, T alpha, T* C, int ldc, T* __restrict__ Cg = nullptr,
                     int ldg = 0, T* __restrict__ tau = nullptr)
{
    const int ntc = (n + 1) / 2;
    const int t = threadIdx.x;
    const int i0 = (t / ntc) * 2, c0 = (t % ntc) * 2;
    const bool act = i0 < m;
    T acc[2][2] = {{T(0), T(0)}, {T(0), T(0)}};
    if (act) {
        int klo, khi;
        k_range<MA, MB>(i0, c0, 2, 2, kk, klo, khi);
#pragma unroll 4
        for (int k = klo; k < khi; ++k) {
            T av[2], bv[2];
#pragma unroll
            for (int r = 0; r < 2; ++r) av[r] = (i0 + r < m) ? op_at<T, TA, MA>(A, lda, i0 + r, k) : T(0);
            const T sc = sB ? sB[k] : T(1);
#pragma unroll
            for (int q = 0; q < 2; ++q) bv[q] = (c0 + q < n) ? sc * op_at<T, TB, MB>(B, ldb, k, c0 + q) : T(0);
#pragma unroll
            for (int r = 0; r < 2; ++r)
#pragma unroll
                for (int q = 0; q < 2; ++q) acc[r][q] += av[r] * bv[q];
        }
    }
    __syncthreads();
    if (act) {
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            const int i = i0 + r;
            if (i >= m) continue;
#pragma unroll
            for (int q = 0; q < 2; ++q) {
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

// Cholesky G = R^T R (b <= 64) with X = R^{-1}: R (upper, zeros below) over
// G, X (upper, zeros below) to Xs.  buf: b scratch entries.
template <typename T>
SKL_DEV void chol_inv_small(T* G, int ldx, int b, const T* __restrict__ mass, T eps, T* Xs, T* buf,
                            int* bad)
{
    chol_smem<T>(G, ldx, b, mass, eps, buf, bad);
    inv_upper_smem<T>(G, ldx, b, Xs, ldx, true, buf);
}

// Modified LU of A (b <= 64) in place (L strict lower, U upper), signs to
// sg, and in Z: L^{-1} (strict lower, unit diagonal implied) and U^{-1}
// (upper).  buf: b scratch entries.
template <typename T>
SKL_DEV void mlu_inv_small(T* A, int ldx, int b, T* sg, T* Z, T* buf)
{
    mlu_smem<T>(A, ldx, b, sg, buf);
    inv_unit_lower_smem<T>(A, ldx, b, Z, ldx);
    inv_upper_smem<T>(A, ldx, b, Z, ldx, false, buf);
}

// b x b workspace layout of the small kernels (row-major, ld = b + 4).
template <typename T>
size_t chol_small_smem_bytes(int b)
{
    return (4 * (size_t)b * (b + 4) + 3 * (size_t)b) * sizeof(T) + 256;
}

// Pass 1: R1 and X1 = R1^{-1} from G1 (column-major b x b, ldg = b).  Sets
// *fail (1 on a Cholesky breakdown, else 0).
template <typename T>
__global__ void __launch_bounds__(kSmallThreads, 1)
k_chol_small1(const T* __restrict__ G, int b, T* __restrict__ R1, T* __restrict__ X1,
              int* __restrict__ fail)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int LDX = b + 4;
    T* S0 = (T*)smem_raw;
    T* S1 = S0 + (size_t)b * LDX;
    T* mass = S1 + (size_t)b * LDX;
    T* buf = mass + b;
    __shared__ int s_bad;
    const T eps = std::is_same<T, float>::value ? T(5.9604645e-08) : T(1.1102230246251565e-16);
    if (threadIdx.x == 0) s_bad = 0;
    for (int e = threadIdx.x; e < b * b; e += kSmallThreads) {
        const int i = e % b, c = e / b;
        S0[i * LDX + c] = G[e];
    }
    for (int k = threadIdx.x; k < b; k += kSmallThreads) mass[k] = G[k * b + k];
    __syncthreads();
    chol_inv_small<T>(S0, LDX, b, mass, eps, S1, buf, &s_bad);
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
    if (*fail) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int LDX = b + 4;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    T* S0 = (T*)smem_raw;                        // R1 -> R = R2 R1
    T* S1 = S0 + (size_t)b * LDX;                // G2 -> R2 -> L^{-1} \ U^{-1}
    T* S2 = S1 + (size_t)b * LDX;                // X2 -> W
    T* S3 = S2 + (size_t)b * LDX;                // Q(0:b,:) -> Q1 -> L \ U
    T* Sg = S3 + (size_t)b * LDX;
    T* mass = Sg + b;
    T* buf = mass + b;
    __shared__ int s_bad;
    const T eps = std::is_same<T, float>::value ? T(5.9604645e-08) : T(1.1102230246251565e-16);
    if (threadIdx.x == 0) s_bad = 0;
    for (int e = threadIdx.x; e < b * b; e += kSmallThreads) {
        const int i = e % b, c = e / b;          // column-major sources
        S1[i * LDX + c] = G[e];
        S3[i * LDX + c] = Q[i + (int64_t)c * ldq];
        const int r = e / b, q = e % b;          // row-major source
        S0[r * LDX + q] = R1g[e];
    }
    for (int k = threadIdx.x; k < b; k += kSmallThreads) mass[k] = T(1);
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
    chol_inv_small<T>(S1, LDX, b, mass, eps, S2, buf, &s_bad);  // R2 over S1, X2 -> S2
    if (s_bad) {
        if (threadIdx.x == 0) *fail = 1;
        return;
    }
    blk_mul<T, false, kMFull, false, kMUpper>(b, b, b, S3, LDX, S2, LDX, nullptr, T(1), S3, LDX);   // Q1 = Q(0:b,:) X2
    blk_mul<T, false, kMUpper, false, kMUpper>(b, b, b, S1, LDX, S0, LDX, nullptr, T(1), S0, LDX);  // R = R2 R1
    mlu_inv_small<T>(S3, LDX, b, Sg, S1, buf);                   // Q1 - S = L U; S1 = L^{-1} \ U^{-1}
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
    k_chol_small1<T><<<1, kSmallThreads, ssm, st>>>(cg, b, cr1, cx1, fail);
    SKL_CUDA(cudaGetLastError());
    SKL_LAUNCHED();
    gemm<T>(false, false, M, b, b, T(1), P, ld, cx1, b, T(0), tmp, M, nullptr, 0, st);
    gemm<T>(true, false, b, b, M, T(1), tmp, M, tmp, M, T(0), cg, b, part, part_cap, st);
    k_chol_small2<T><<<1, kSmallThreads, ssm, st>>>(cg, b, cr1, tmp, M, A, ld, j0, V, ldv, Tm, ldt,
                                                    tau, cw, fail);
    SKL_CUDA(cudaGetLastError());
    SKL_LAUNCHED();
    gemm<T>(false, false, M - b, b, b, T(1), tmp + b, M, cw, b, T(0), V + b, ldv, nullptr, 0, st);
    dim3 gc((unsigned)std::max<int64_t>(1, std::min<int64_t>((M - b + 255) / 256, 64)), b);
    k_chol_copy_down<T><<<gc, 256, 0, st>>>(V, ldv, A, ld, j0, M, b, fail);
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
