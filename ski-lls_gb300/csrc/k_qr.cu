// k_qr.cu -- randomized column-pivoted Householder QR of the sketch S*A.
//
// Algorithm: HQRRP (Martinsson, Quintana-Orti, Heavner, van de Geijn), as the
// reference uses it through dgeqp4_INT / NoFLA_HQRRP_WY_blk_var4_INT
// (hqrrp/lapack_compatible_sources/NoFLA_HQRRP_WY_blk_var4_skint.c:313-582):
//
//   Y = G*A with G Gaussian (nb+pp) x m;
//   for each block of nb columns:
//     1. QR with column pivoting of the small sample Y(:, j:) picks nb pivots
//        (skint.c:501-518), applied to A, Y and jpvt;
//     2. QR with pivoting of the panel A(j:m, j:j+nb) and its T factor
//        (skint.c:530-535);
//     3. trailing update A(j:m, j+nb:) <- Q^T A(j:m, j+nb:)  (skint.c:540-551);
//     4. Y downdate and G <- G Q  (skint.c:554-568, :627-718).
//
// GB300 mapping.  Steps 1 and 2 are chains of rank-1 steps, each needing a
// reduction over the whole column set or row set.  Each runs as ONE cluster
// of 16 CTAs with the operand resident in the cluster's shared memory
// (distributed shared memory): a reduction is a write to local shared memory,
// a hardware cluster barrier (~0.25 us) and DSMEM loads, instead of a
// grid-wide barrier (~2 us) or a kernel launch per column.  Steps 3-4 are
// GEMMs.  The sample G is drawn on the device from a counter-based generator
// (the reference draws it from srand(12) + Marsaglia's polar method,
// skint.c:390,584-624; the pivots of a randomized QR are not expected to be
// reproduced bit for bit, only the solution).
//
// Also applies Q^T to the sketched right-hand side during the factorization
// (the reference does it afterwards with dormqr,
// src/ls_dense_hashing_blendenpik.cpp:70-76).
#include <cmath>
#include <cstdio>

#include "skl_internal.hpp"
#include "common.cuh"
#include "k_gemm.cuh"

namespace skl {

constexpr int kQrThreads = 512;
constexpr int kQrWarps = kQrThreads / 32;
constexpr int kCluster = 16;
constexpr int kPP = 16;          // over-sampling rows of the sample Y
constexpr int kMaxNb = 64;

// ------------------------------------------------------------- Gaussian --
SKL_DEV unsigned long long splitmix64(unsigned long long x)
{
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

template <typename T>
__global__ void k_gaussian(T* __restrict__ G, int64_t count, unsigned long long seed)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count;
         i += (int64_t)gridDim.x * blockDim.x) {
        unsigned long long r = splitmix64(seed ^ splitmix64((unsigned long long)i));
        double u1 = ((r >> 11) + 1.0) * (1.0 / 9007199254740993.0);   // (0,1]
        unsigned long long r2 = splitmix64(r);
        double u2 = (r2 >> 11) * (1.0 / 9007199254740992.0);
        G[i] = (T)(sqrt(-2.0 * log(u1)) * cospi(2.0 * u2));
    }
}

// ------------------------------------------------------ Householder math --
// dlarfg semantics: given alpha and sigma2 = ||x||^2 of the part below,
// beta = -sign(alpha) sqrt(alpha^2 + sigma2), tau = (beta - alpha)/beta,
// v = x / (alpha - beta).  sigma2 == 0 gives tau = 0 (H = I), beta = alpha.
template <typename T>
SKL_DEV void householder(T alpha, T sigma2, T& beta, T& tau, T& scale)
{
    if (sigma2 <= T(0)) {
        beta = alpha;
        tau = T(0);
        scale = T(0);
        return;
    }
    T nrm = t_sqrt(alpha * alpha + sigma2);
    beta = alpha >= T(0) ? -nrm : nrm;
    tau = (beta - alpha) / beta;
    scale = T(1) / (alpha - beta);
}

// ------------------------------------------------------------ Y-QRP -----
// QR with column pivoting of Y(:, j0:j0+N) (nbp x N) for b steps; writes the
// selected columns (relative indices) in selection order to sel[0..b).
template <typename T>
struct YqrpSmem {
    // layout offsets in the dynamic shared buffer
    static size_t bytes(int nbp, int cn)
    {
        size_t s = (size_t)nbp * cn * sizeof(T);          // Ys
        s += (size_t)cn * sizeof(T);                       // nrm
        s += (size_t)cn;                                   // taken
        s = (s + 15) & ~(size_t)15;
        s += 2 * (size_t)nbp * sizeof(T);                  // cand_col[2]
        s += (size_t)nbp * sizeof(T);                      // v
        s += 2 * sizeof(T) + 2 * sizeof(int) + 64;         // cand val/idx
        return s + 256;
    }
};

template <typename T>
__global__ void __launch_bounds__(kQrThreads)
k_yqrp(const T* __restrict__ Y, int ldy, int nbp, int j0, int N, int b, int* __restrict__ sel)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const unsigned crank = cluster_ctarank();
    const int cn = (N + kCluster - 1) / kCluster;
    const int c0 = (int)crank * cn;
    const int ncols = max(0, min(cn, N - c0));
    T* Ys = (T*)smem_raw;
    T* nrm = Ys + (size_t)nbp * cn;
    unsigned char* taken = (unsigned char*)(nrm + cn);
    size_t off = ((size_t)nbp * cn * sizeof(T) + cn * sizeof(T) + cn + 15) & ~(size_t)15;
    T* cand_col = (T*)(smem_raw + off);          // [2][nbp]
    T* v = cand_col + 2 * nbp;                    // [nbp]
    T* cand_val = v + nbp;                        // [2]
    int* cand_idx = (int*)(cand_val + 2);         // [2]
    __shared__ T s_red_v[kQrWarps];
    __shared__ int s_red_i[kQrWarps];
    __shared__ T s_tau;

    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    for (int e = tid; e < nbp * ncols; e += kQrThreads) {
        int r = e % nbp, c = e / nbp;
        Ys[r + (size_t)c * nbp] = Y[r + (int64_t)(j0 + c0 + c) * ldy];
    }
    for (int c = tid; c < cn; c += kQrThreads) taken[c] = (c < ncols) ? 0 : 1;
    __syncthreads();
    for (int c = wid; c < ncols; c += kQrWarps) {
        T s = T(0);
        for (int r = lane; r < nbp; r += 32) { T y = Ys[r + (size_t)c * nbp]; s += y * y; }
        s = warp_sum(s);
        if (lane == 0) nrm[c] = s;
    }
    __syncthreads();

    for (int s = 0; s < b; ++s) {
        const int p = s & 1;
        // (a) local argmax (largest norm; ties -> smallest index)
        T bv = T(-1);
        int bi = -1;
        for (int c = tid; c < ncols; c += kQrThreads) {
            if (!taken[c] && nrm[c] > bv) { bv = nrm[c]; bi = c; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            T ov = __shfl_xor_sync(0xffffffffu, bv, o);
            int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ov > bv || (ov == bv && oi >= 0 && (bi < 0 || oi < bi))) { bv = ov; bi = oi; }
        }
        if (lane == 0) { s_red_v[wid] = bv; s_red_i[wid] = bi; }
        __syncthreads();
        if (tid == 0) {
            T v0 = T(-1);
            int i0 = -1;
            for (int w = 0; w < kQrWarps; ++w) {
                T ov = s_red_v[w];
                int oi = s_red_i[w];
                if (ov > v0 || (ov == v0 && oi >= 0 && (i0 < 0 || oi < i0))) { v0 = ov; i0 = oi; }
            }
            cand_val[p] = v0;
            cand_idx[p] = (i0 >= 0) ? c0 + i0 : -1;
            s_red_i[0] = i0;
        }
        __syncthreads();
        {
            int li = s_red_i[0];
            for (int r = tid; r < nbp; r += kQrThreads)
                cand_col[p * nbp + r] = (li >= 0) ? Ys[r + (size_t)li * nbp] : T(0);
        }
        cluster_sync();
        // (c) global winner
        if (wid == 0) {
            T ov = T(-1);
            int oi = -1, orank = 0;
            if (lane < kCluster) {
                ov = dsmem_ld(&cand_val[p], lane);
                oi = dsmem_ld_s32(&cand_idx[p], lane);
                orank = lane;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                T xv = __shfl_xor_sync(0xffffffffu, ov, o);
                int xi = __shfl_xor_sync(0xffffffffu, oi, o);
                int xr = __shfl_xor_sync(0xffffffffu, orank, o);
                if (xv > ov || (xv == ov && xi >= 0 && (oi < 0 || xi < oi))) { ov = xv; oi = xi; orank = xr; }
            }
            // winner column into v (rows s..nbp-1)
            for (int r = s + lane; r < nbp; r += 32) v[r] = dsmem_ld(&cand_col[p * nbp + r], orank);
            __syncwarp();
            T sg = T(0);
            for (int r = s + 1 + lane; r < nbp; r += 32) sg += v[r] * v[r];
            sg = warp_sum(sg);
            T beta, tau, scale;
            householder(v[s], sg, beta, tau, scale);
            __syncwarp();
            for (int r = s + 1 + lane; r < nbp; r += 32) v[r] *= scale;
            if (lane == 0) {
                v[s] = T(1);
                s_tau = tau;
                if (crank == 0) sel[s] = oi;
                if (oi >= c0 && oi < c0 + ncols) taken[oi - c0] = 1;
            }
        }
        __syncthreads();
        const T tau = s_tau;
        // (d) apply H = I - tau v v^T to the untaken local columns, new norms
        for (int c = wid; c < ncols; c += kQrWarps) {
            if (taken[c]) continue;
            T* col = Ys + (size_t)c * nbp;
            T w = T(0);
            for (int r = s + lane; r < nbp; r += 32) w += v[r] * col[r];
            w = warp_sum(w) * tau;
            T ss = T(0);
            for (int r = s + lane; r < nbp; r += 32) {
                T y = col[r] - w * v[r];
                col[r] = y;
                if (r > s) ss += y * y;
            }
            ss = warp_sum(ss);
            if (lane == 0) nrm[c] = ss;
        }
        __syncthreads();
    }
    cluster_sync();   // keep shared memory alive until every CTA finished reading it
}

// -------------------------------------------------- column permutation --
// Moves the selected columns (sel, relative to j0) to positions j0..j0+b-1;
// the columns they displace fill the vacated positions in increasing order.
// plan: src[t] for t in [0, 2b): dest position dst[t] (relative) <- src.
__global__ void k_perm_plan(const int* __restrict__ sel, int b, int* __restrict__ plan_src,
                            int* __restrict__ plan_dst, int* __restrict__ plan_n)
{
    __shared__ int in_low[kMaxNb];
    __shared__ int high_sel[kMaxNb];
    __shared__ int nhigh;
    const int t = threadIdx.x;
    if (t < kMaxNb) in_low[t] = 0;
    if (t == 0) nhigh = 0;
    __syncthreads();
    if (t < b) {
        int s = sel[t];
        if (s < b) in_low[s] = 1;
    }
    __syncthreads();
    if (t == 0) {
        // deterministic serial pass over <= 64 entries
        int nh = 0;
        for (int q = 0; q < b; ++q) if (sel[q] >= b) high_sel[nh++] = sel[q];
        // sort vacated positions ascending (insertion sort, <= 64)
        for (int a = 1; a < nh; ++a) {
            int x = high_sel[a], c = a - 1;
            while (c >= 0 && high_sel[c] > x) { high_sel[c + 1] = high_sel[c]; --c; }
            high_sel[c + 1] = x;
        }
        nhigh = nh;
        int n = 0;
        for (int q = 0; q < b; ++q) {           // selected -> front
            plan_src[n] = sel[q];
            plan_dst[n] = q;
            ++n;
        }
        int h = 0;
        for (int pos = 0; pos < b; ++pos) {      // displaced -> vacated
            if (!in_low[pos]) {
                plan_src[n] = pos;
                plan_dst[n] = high_sel[h++];
                ++n;
            }
        }
        *plan_n = n;
    }
}

// Copy the planned source columns of X (rows x cols, ld) into tmp, then
// write them to their destinations.  Also permutes jpvt.
template <typename T>
__global__ void k_perm_gather(const T* __restrict__ X, int64_t ld, int rows, int j0,
                              const int* __restrict__ plan_src, const int* __restrict__ plan_n,
                              T* __restrict__ tmp)
{
    const int q = blockIdx.y;
    if (q >= *plan_n) return;
    const T* src = X + (int64_t)(j0 + plan_src[q]) * ld;
    T* dst = tmp + (int64_t)q * rows;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x)
        dst[r] = src[r];
}

template <typename T>
__global__ void k_perm_scatter(T* __restrict__ X, int64_t ld, int rows, int j0,
                               const int* __restrict__ plan_dst, const int* __restrict__ plan_n,
                               const T* __restrict__ tmp)
{
    const int q = blockIdx.y;
    if (q >= *plan_n) return;
    T* dst = X + (int64_t)(j0 + plan_dst[q]) * ld;
    const T* src = tmp + (int64_t)q * rows;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x)
        dst[r] = src[r];
}

__global__ void k_perm_ints(int* __restrict__ jpvt, int j0, const int* __restrict__ plan_src,
                            const int* __restrict__ plan_dst, const int* __restrict__ plan_n)
{
    __shared__ int vals[2 * kMaxNb];
    const int n = *plan_n;
    for (int q = threadIdx.x; q < n; q += blockDim.x) vals[q] = jpvt[j0 + plan_src[q]];
    __syncthreads();
    for (int q = threadIdx.x; q < n; q += blockDim.x) jpvt[j0 + plan_dst[q]] = vals[q];
}

// ------------------------------------------------------------- panel ----
// Pivoted Householder QR of the panel P = A(j0:m, j0:j0+b) held in the
// cluster's shared memory (CTA c owns panel rows [c*R, c*R+R)).
template <typename T>
size_t panel_smem_bytes(int R, int b)
{
    size_t s = (size_t)R * b * sizeof(T);       // Ps
    s += 4 * (size_t)kMaxNb * sizeof(T);        // red1, red2, rowS, nrm2
    s += (size_t)kMaxNb * kMaxNb * sizeof(T);   // gram partial
    s += (size_t)kMaxNb * kMaxNb * sizeof(T);   // T (rank 0 only)
    s += 2 * (size_t)kMaxNb * sizeof(int);      // piv history
    return s + 512;
}

template <typename T>
__global__ void __launch_bounds__(kQrThreads)
k_panel(T* __restrict__ A, int64_t ld, int j0, int M, int b, int R, T* __restrict__ tau_out,
        T* __restrict__ Tout, int ldt, T* __restrict__ V, int64_t ldv, int* __restrict__ jpvt,
        T* __restrict__ Y, int ldy, int nbp, int pivot_panel)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const unsigned crank = cluster_ctarank();
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int r0 = (int)crank * R;                      // first panel row owned
    const int nr = max(0, min(R, M - r0));              // rows owned
    T* Ps = (T*)smem_raw;                               // [b][R] column-major
    T* red1 = Ps + (size_t)R * b;
    T* red2 = red1 + kMaxNb;
    T* rowS = red2 + kMaxNb;
    T* nrm2 = rowS + kMaxNb;
    T* gram = nrm2 + kMaxNb;
    T* Tl = gram + kMaxNb * kMaxNb;
    int* pivh = (int*)(Tl + kMaxNb * kMaxNb);
    __shared__ T s_beta, s_tau, s_scale;
    __shared__ int s_piv;

    // load the panel rows
    for (int e = tid; e < nr * b; e += kQrThreads) {
        int lr = e % nr, c = e / nr;
        Ps[lr + (size_t)c * R] = A[(int64_t)(j0 + r0 + lr) + (int64_t)(j0 + c) * ld];
    }
    __syncthreads();
    // initial partial norms over rows > 0 and row 0 values
    for (int c = wid; c < b; c += kQrWarps) {
        T ss = T(0);
        for (int lr = lane; lr < nr; lr += 32) {
            int g = r0 + lr;
            T x = Ps[lr + (size_t)c * R];
            if (g > 0) ss += x * x;
            else rowS[c] = x;
        }
        ss = warp_sum(ss);
        if (lane == 0) red1[c] = ss;
    }
    const int steps = min(b, M);
    for (int s = 0; s < steps; ++s) {
        const unsigned own = (unsigned)(s / R);          // CTA holding panel row s
        cluster_sync();                                  // (A) red1, rowS published
        // full column norms for columns s..b-1
        for (int c = s + wid; c < b; c += kQrWarps) {
            T x = T(0);
            if (lane < kCluster) x = dsmem_ld(&red1[c], lane);
            x = warp_sum(x);
            if (lane == 0) {
                T a = dsmem_ld(&rowS[c], own);
                nrm2[c] = x + a * a;
                red2[c] = x;   // below-row-s part kept for sigma^2 (local copy)
            }
        }
        __syncthreads();
        if (tid == 0) {
            int piv = s;
            T best = nrm2[s];
            if (pivot_panel)
                for (int c = s + 1; c < b; ++c)
                    if (nrm2[c] > best) { best = nrm2[c]; piv = c; }
            T alpha = dsmem_ld(&rowS[piv], own);
            T beta, tau, scale;
            householder(alpha, red2[piv], beta, tau, scale);
            s_piv = piv;
            s_beta = beta;
            s_tau = tau;
            s_scale = scale;
            pivh[s] = piv;
        }
        __syncthreads();
        const int piv = s_piv;
        const T tau = s_tau, scale = s_scale;
        if (piv != s) {
            for (int lr = tid; lr < nr; lr += kQrThreads) {
                T a = Ps[lr + (size_t)s * R], c = Ps[lr + (size_t)piv * R];
                Ps[lr + (size_t)s * R] = c;
                Ps[lr + (size_t)piv * R] = a;
            }
        }
        __syncthreads();
        // v: scale rows > s of column s; row s keeps beta (R_ss), v_s = 1
        for (int lr = tid; lr < nr; lr += kQrThreads) {
            int g = r0 + lr;
            if (g > s) Ps[lr + (size_t)s * R] *= scale;
            else if (g == s) Ps[lr + (size_t)s * R] = s_beta;
        }
        __syncthreads();
        // partial w_c = sum_{rows >= s} v_r P[r][c], c > s
        const int lr_s = max(0, s - r0);   // first local row with g >= s
        for (int c = s + 1 + wid; c < b; c += kQrWarps) {
            T acc = T(0);
            for (int lr = lr_s + lane; lr < nr; lr += 32) {
                int g = r0 + lr;
                T vv = (g == s) ? T(1) : Ps[lr + (size_t)s * R];
                acc += vv * Ps[lr + (size_t)c * R];
            }
            acc = warp_sum(acc);
            if (lane == 0) red2[c] = acc;
        }
        cluster_sync();                                  // (B) red2 published
        for (int c = s + 1 + wid; c < b; c += kQrWarps) {
            T w = T(0);
            if (lane < kCluster) w = dsmem_ld(&red2[c], lane);
            w = warp_sum(w) * tau;
            T ss = T(0);
            for (int lr = lr_s + lane; lr < nr; lr += 32) {
                int g = r0 + lr;
                T vv = (g == s) ? T(1) : Ps[lr + (size_t)s * R];
                T x = Ps[lr + (size_t)c * R] - w * vv;
                Ps[lr + (size_t)c * R] = x;
                if (g > s + 1) ss += x * x;
                else if (g == s + 1) rowS[c] = x;
            }
            ss = warp_sum(ss);
            if (lane == 0) red1[c] = ss;
        }
        if (tid == 0 && crank == 0) tau_out[j0 + s] = tau;
        __syncthreads();
    }
    // Gram matrix of V (unit lower trapezoid) for the T factor: one warp per
    // (a, c) pair, lanes over rows.
    for (int e = wid; e < b * b; e += kQrWarps) {
        int a = e % b, c = e / b;
        T acc = T(0);
        if (a < c) {
            int lr0 = max(0, c - r0);          // V[:,c] is zero above row c
            for (int lr = lr0 + lane; lr < nr; lr += 32) {
                int g = r0 + lr;
                T vc = (g == c) ? T(1) : Ps[lr + (size_t)c * R];
                T va = Ps[lr + (size_t)a * R];  // g >= c > a
                acc += va * vc;
            }
            acc = warp_sum(acc);
        }
        if (lane == 0) gram[a + c * kMaxNb] = acc;
    }
    cluster_sync();
    if (crank == 0) {
        // sum the partial Gram matrices
        for (int e = tid; e < b * b; e += kQrThreads) {
            int a = e % b, c = e / b;
            if (a >= c) continue;
            T acc = T(0);
            for (int q = 0; q < kCluster; ++q) acc += dsmem_ld(&gram[a + c * kMaxNb], q);
            Tl[a + c * kMaxNb] = acc;     // holds V_a^T V_c for a < c (temporarily)
        }
        __syncthreads();
        // T (dlarft forward/columnwise): T_ii = tau_i,
        // T(0:i, i) = -tau_i * T(0:i, 0:i) * (V(:,0:i)^T v_i)
        __shared__ T col[kMaxNb];
        for (int i = 0; i < b; ++i) {
            T ti = tau_out[j0 + i];
            if (tid < i) col[tid] = Tl[tid + i * kMaxNb];
            __syncthreads();
            if (tid < i) {
                T acc = T(0);
                for (int c = tid; c < i; ++c) acc += gram[tid + c * kMaxNb] * col[c];
                // gram[] now used as the T storage (upper part), see below
                Tl[tid + i * kMaxNb] = -ti * acc;
            }
            __syncthreads();
            if (tid == 0) gram[i + i * kMaxNb] = ti;
            if (tid < i) gram[tid + i * kMaxNb] = Tl[tid + i * kMaxNb];
            __syncthreads();
        }
        for (int e = tid; e < b * b; e += kQrThreads) {
            int a = e % b, c = e / b;
            Tout[a + (int64_t)c * ldt] = (a <= c) ? gram[a + c * kMaxNb] : T(0);
        }
    }
    cluster_sync();   // other CTAs' Gram partials must stay alive until read
    // write back panel: R (upper) + V (below) into A; explicit V into V buffer
    for (int e = tid; e < nr * b; e += kQrThreads) {
        int lr = e % nr, c = e / nr;
        int g = r0 + lr;
        T x = Ps[lr + (size_t)c * R];
        A[(int64_t)(j0 + g) + (int64_t)(j0 + c) * ld] = x;
        V[(int64_t)g + (int64_t)c * ldv] = (g > c) ? x : (g == c ? T(1) : T(0));
    }
    // apply the panel's column swaps to rows above the panel, to Y and jpvt
    const int nabove = j0;
    for (int row = (int)crank * kQrThreads + tid; row < nabove + nbp + 1;
         row += kCluster * kQrThreads) {
        if (row < nabove) {
            T* base = A + row;
            for (int s = 0; s < steps; ++s) {
                int p = pivh[s];
                if (p != s) {
                    T a = base[(int64_t)(j0 + s) * ld];
                    base[(int64_t)(j0 + s) * ld] = base[(int64_t)(j0 + p) * ld];
                    base[(int64_t)(j0 + p) * ld] = a;
                }
            }
        } else if (row < nabove + nbp) {
            if (Y) {
                T* base = Y + (row - nabove);
                for (int s = 0; s < steps; ++s) {
                    int p = pivh[s];
                    if (p != s) {
                        T a = base[(int64_t)(j0 + s) * ldy];
                        base[(int64_t)(j0 + s) * ldy] = base[(int64_t)(j0 + p) * ldy];
                        base[(int64_t)(j0 + p) * ldy] = a;
                    }
                }
            }
        } else {
            for (int s = 0; s < steps; ++s) {
                int p = pivh[s];
                if (p != s) {
                    int a = jpvt[j0 + s];
                    jpvt[j0 + s] = jpvt[j0 + p];
                    jpvt[j0 + p] = a;
                }
            }
        }
    }
}

// ------------------------------------------------- Q^T c for one panel --
// c(j0:m) <- (I - V T^T V^T) c(j0:m), FP64 accumulation.
template <typename T>
__global__ void k_qt_w(const T* __restrict__ V, int64_t ldv, int M, int b,
                       const double* __restrict__ c, double* __restrict__ w)
{
    __shared__ double red[kQrWarps];
    const int a = blockIdx.x;
    double acc = 0.0;
    for (int r = threadIdx.x; r < M; r += blockDim.x) acc = fma((double)V[r + (int64_t)a * ldv], c[r], acc);
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) w[a] = acc;
}

template <typename T>
__global__ void k_qt_update(const T* __restrict__ V, int64_t ldv, int M, int b,
                            const T* __restrict__ Tm, int ldt, const double* __restrict__ w,
                            double* __restrict__ c)
{
    __shared__ double z[kMaxNb];
    // z = T^T w
    if (threadIdx.x < b) {
        int i = threadIdx.x;
        double acc = 0.0;
        for (int a = 0; a <= i; ++a) acc = fma((double)Tm[a + (int64_t)i * ldt], w[a], acc);
        z[i] = acc;
    }
    __syncthreads();
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < M; r += gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int a = 0; a < b; ++a) acc = fma((double)V[r + (int64_t)a * ldv], z[a], acc);
        c[r] -= acc;
    }
}

template <typename T>
__global__ void k_copy_block(const T* __restrict__ src, int64_t lds, T* __restrict__ dst,
                             int64_t ldd, int rows, int cols)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < rows * cols; e += gridDim.x * blockDim.x) {
        int r = e % rows, c = e / rows;
        dst[r + (int64_t)c * ldd] = src[r + (int64_t)c * lds];
    }
}

__global__ void k_iota_int(int* v, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = i;
}

// ------------------------------------------------------------ host side --
struct QrPlan {
    int nb, nbp, R;
};

template <typename T>
static QrPlan qr_plan(int64_t m, int64_t d)
{
    QrPlan p;
    p.R = (int)((m + kCluster - 1) / kCluster);
    int nb = kMaxNb;
    size_t budget = 200 * 1024;
    while (nb > 8 && panel_smem_bytes<T>(p.R, nb) > budget) nb -= 8;
    if (panel_smem_bytes<T>(p.R, nb) > budget)
        fail(SKL_ERR_INVALID, "cpqr: sketch has too many rows for the shared-memory panel (m=" +
                                  std::to_string(m) + ")");
    p.nb = nb;
    p.nbp = nb + kPP;
    int64_t cn = (d + kCluster - 1) / kCluster;
    if (YqrpSmem<T>::bytes(p.nbp, (int)cn) > budget)
        fail(SKL_ERR_INVALID, "cpqr: too many columns for the shared-memory sample QRP (d=" +
                                  std::to_string(d) + ")");
    return p;
}

template <typename T>
struct QrBuffers {
    T *G, *Y, *V, *Tm, *W, *Z, *GU, *GUT, *Bm, *part, *tmp;
    int *sel, *plan_src, *plan_dst, *plan_n;
    double *qw;
    int64_t part_cap, tmp_rows;
};

template <typename T>
static QrBuffers<T> qr_carve(void* work, int64_t m, int64_t d, const QrPlan& p, size_t* total)
{
    char* base = (char*)work;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        void* r = base ? base + off : nullptr;
        off += (bytes + 255) & ~(size_t)255;
        return r;
    };
    QrBuffers<T> B;
    B.G = (T*)take((size_t)p.nbp * m * sizeof(T));
    B.Y = (T*)take((size_t)p.nbp * d * sizeof(T));
    B.V = (T*)take((size_t)m * p.nb * sizeof(T));
    B.Tm = (T*)take((size_t)p.nb * p.nb * sizeof(T));
    B.W = (T*)take((size_t)p.nb * d * sizeof(T));
    B.Z = (T*)take((size_t)p.nb * d * sizeof(T));
    B.GU = (T*)take((size_t)p.nbp * p.nb * sizeof(T));
    B.GUT = (T*)take((size_t)p.nbp * p.nb * sizeof(T));
    B.Bm = (T*)take((size_t)p.nbp * p.nb * sizeof(T));
    int64_t cap = (int64_t)p.nbp * (d > m ? d : m) * 8;
    if (cap < (int64_t)1 << 20) cap = (int64_t)1 << 20;
    B.part_cap = cap;
    B.part = (T*)take((size_t)cap * sizeof(T));
    B.tmp_rows = m > p.nbp ? m : p.nbp;
    B.tmp = (T*)take((size_t)B.tmp_rows * 2 * p.nb * sizeof(T));
    B.sel = (int*)take(kMaxNb * sizeof(int));
    B.plan_src = (int*)take(2 * kMaxNb * sizeof(int));
    B.plan_dst = (int*)take(2 * kMaxNb * sizeof(int));
    B.plan_n = (int*)take(sizeof(int));
    B.qw = (double*)take(kMaxNb * sizeof(double));
    if (total) *total = off;
    return B;
}

template <typename T>
size_t cpqr_workspace_bytes(int64_t m, int64_t d)
{
    QrPlan p = qr_plan<T>(m, d);
    size_t total = 0;
    qr_carve<T>(nullptr, m, d, p, &total);
    return total;
}

template <typename T>
static void launch_cluster(const void* fn, dim3 block, size_t smem, cudaStream_t st, void** args)
{
    SKL_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    SKL_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kCluster, 1, 1);
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = kCluster;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    SKL_CUDA(cudaLaunchKernelExC(&cfg, fn, args));
    SKL_LAUNCHED();
}

template <typename T>
static void qr_core(T* A, int64_t m, int64_t d, int64_t ld, int* jpvt, T* tau, void* work,
                    cudaStream_t st, double* c, bool pivoting)
{
    QrPlan p = qr_plan<T>(m, d);
    QrBuffers<T> B = qr_carve<T>(work, m, d, p, nullptr);
    const int nb = p.nb, nbp = p.nbp;
    const int64_t mn = m < d ? m : d;
    k_iota_int<<<(unsigned)((d + 255) / 256), 256, 0, st>>>(jpvt, (int)d);
    SKL_LAUNCHED();
    if (pivoting) {
        int64_t cnt = (int64_t)nbp * m;
        k_gaussian<T><<<(unsigned)((cnt + 255) / 256 < 2048 ? (cnt + 255) / 256 : 2048), 256, 0, st>>>(
            B.G, cnt, 0x5eed000000000012ull);
        SKL_LAUNCHED();
        gemm<T>(false, false, nbp, (int)d, (int)m, T(1), B.G, nbp, A, ld, T(0), B.Y, nbp, B.part,
                B.part_cap, st);
    }
    const size_t ysm_max = YqrpSmem<T>::bytes(nbp, (int)((d + kCluster - 1) / kCluster));
    const size_t psm = panel_smem_bytes<T>(p.R, nb);
    for (int64_t j = 0; j < mn; j += nb) {
        const int b = (int)std::min<int64_t>(nb, std::min<int64_t>(d - j, m - j));
        const bool last = (j + nb >= m) || (j + nb >= d);
        const int M = (int)(m - j);
        const int N = (int)(d - j);
        trace_phase(st, "qr: panel start");
        if (pivoting && !last) {
            int jj = (int)j;
            int ldy = nbp;
            const T* Yc = B.Y;
            int* sel = B.sel;
            void* args[] = {(void*)&Yc, &ldy, (void*)&nbp, &jj, (void*)&N, (void*)&b, &sel};
            launch_cluster<T>((const void*)k_yqrp<T>, dim3(kQrThreads), ysm_max, st, args);
            trace_phase(st, "qr: yqrp");
            k_perm_plan<<<1, kMaxNb, 0, st>>>(B.sel, b, B.plan_src, B.plan_dst, B.plan_n);
            SKL_LAUNCHED();
            dim3 gA((unsigned)std::min<int64_t>((m + 255) / 256, 64), 2 * b);
            k_perm_gather<T><<<gA, 256, 0, st>>>(A, ld, (int)m, jj, B.plan_src, B.plan_n, B.tmp);
            k_perm_scatter<T><<<gA, 256, 0, st>>>(A, ld, (int)m, jj, B.plan_dst, B.plan_n, B.tmp);
            dim3 gY(1, 2 * b);
            k_perm_gather<T><<<gY, 128, 0, st>>>(B.Y, nbp, nbp, jj, B.plan_src, B.plan_n, B.tmp);
            k_perm_scatter<T><<<gY, 128, 0, st>>>(B.Y, nbp, nbp, jj, B.plan_dst, B.plan_n, B.tmp);
            k_perm_ints<<<1, 128, 0, st>>>(jpvt, jj, B.plan_src, B.plan_dst, B.plan_n);
            for (int q = 0; q < 5; ++q) SKL_LAUNCHED();
        }
        {
            // panel: with pivoting=false the panel keeps its column order
            int jj = (int)j, R = p.R, ldt = nb, nbpp = nbp;
            int64_t ldv = m;
            T* tau_p = tau;
            T* Tm = B.Tm;
            T* V = B.V;
            T* Yp = pivoting ? B.Y : nullptr;
            int ldy = nbp;
            int pp = pivoting ? 1 : 0;
            void* args[] = {&A, &ld, &jj, (void*)&M, (void*)&b, &R, &tau_p, &Tm, &ldt, &V,
                            &ldv, &jpvt, &Yp, &ldy, &nbpp, &pp};
            launch_cluster<T>((const void*)k_panel<T>, dim3(kQrThreads), psm, st, args);
            trace_phase(st, "qr: panel");
        }
        if (c) {
            k_qt_w<T><<<b, 256, 0, st>>>(B.V, m, M, b, c + j, B.qw);
            k_qt_update<T><<<(unsigned)std::min<int64_t>((M + 255) / 256, 256), 256, 0, st>>>(
                B.V, m, M, b, B.Tm, nb, B.qw, c + j);
            SKL_LAUNCHED();
            SKL_LAUNCHED();
        }
        const int N2 = N - b;
        if (N2 > 0) {
            T* Atr = A + j + (j + b) * ld;
            // W = V^T A_trail ; Z = T^T W ; A_trail -= V Z
            gemm<T>(true, false, b, N2, M, T(1), B.V, m, Atr, ld, T(0), B.W, b, B.part,
                    B.part_cap, st);
            gemm<T>(true, false, b, N2, b, T(1), B.Tm, nb, B.W, b, T(0), B.Z, b, nullptr, 0, st);
            gemm<T>(false, false, M, N2, b, T(-1), B.V, m, B.Z, b, T(1), Atr, ld, nullptr, 0, st);
        }
        if (pivoting && !last) {
            T* Gj = B.G + j * nbp;
            // GU = G(:, j:m) V ; GUT = GU T ; B = G1 - GUT U11^T ; Y2 -= B R12 ; G(:, j:m) -= GUT V^T
            gemm<T>(false, false, nbp, b, M, T(1), Gj, nbp, B.V, m, T(0), B.GU, nbp, B.part,
                    B.part_cap, st);
            gemm<T>(false, false, nbp, b, b, T(1), B.GU, nbp, B.Tm, nb, T(0), B.GUT, nbp, nullptr,
                    0, st);
            k_copy_block<T><<<16, 256, 0, st>>>(Gj, nbp, B.Bm, nbp, nbp, b);
            SKL_LAUNCHED();
            gemm<T>(false, true, nbp, b, b, T(-1), B.GUT, nbp, B.V, m, T(1), B.Bm, nbp, nullptr, 0,
                    st);
            if (N2 > 0)
                gemm<T>(false, false, nbp, N2, b, T(-1), B.Bm, nbp, A + j + (j + b) * ld, ld, T(1),
                        B.Y + (j + b) * nbp, nbp, nullptr, 0, st);
            gemm<T>(false, true, nbp, M, b, T(-1), B.GUT, nbp, B.V, m, T(1), Gj, nbp, nullptr, 0,
                    st);
        }
    }
}

template <typename T>
void cpqr(T* A, int64_t m, int64_t d, int64_t ld, int* jpvt, T* tau, void* work, unsigned* status,
          cudaStream_t st, double* c, int pivoting)
{
    (void)status;
    qr_core<T>(A, m, d, ld, jpvt, tau, work, st, c, pivoting != 0);
}

template void cpqr<float>(float*, int64_t, int64_t, int64_t, int*, float*, void*, unsigned*,
                          cudaStream_t, double*, int);
template void cpqr<double>(double*, int64_t, int64_t, int64_t, int*, double*, void*, unsigned*,
                           cudaStream_t, double*, int);
template size_t cpqr_workspace_bytes<float>(int64_t, int64_t);
template size_t cpqr_workspace_bytes<double>(int64_t, int64_t);

}  // namespace skl
