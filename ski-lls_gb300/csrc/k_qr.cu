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
// GB300 mapping.  Step 1 is a chain of rank-1 steps, each needing a reduction
// over the whole column set; it runs as ONE cluster of 16 CTAs with the sample
// resident in the cluster's shared memory: each CTA pushes its candidate to
// every CTA with remote shared-memory stores, then one hardware cluster
// barrier (~0.25 us) replaces a grid-wide barrier (~2 us) or a launch per
// column.  Step 2 on the FP32 path is CholeskyQR2 of the panel in the order
// the sample chose (GEMMs over the whole GPU plus small one-CTA kernels, in
// k_qr_chol.cu), falling back to the pivoted cluster panel (k_panel) when the
// Cholesky breaks down; the FP64 path uses k_panel.  Steps 3-4 are GEMMs, the
// sample work (step 4 and the next step 1) on a second, high-priority stream
// overlapping the trailing update.  The sample G is drawn on the device from a counter-based generator
// (the reference draws it from srand(12) + Marsaglia's polar method,
// skint.c:390,584-624; the pivots of a randomized QR are not expected to be
// reproduced bit for bit, only the solution).
//
// Also applies Q^T to the sketched right-hand side during the factorization
// (the reference does it afterwards with dormqr,
// src/ls_dense_hashing_blendenpik.cpp:70-76).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "skl_internal.hpp"
#include "launch.cuh"
#include "common.cuh"
#include "k_gemm.cuh"

namespace skl {

constexpr int kQrThreads = 512;
constexpr int kYThreads = 512;    // sample QRP block
constexpr int kYWarps = kYThreads / 32;
constexpr int kQrWarps = kQrThreads / 32;
constexpr int kCluster = 16;
constexpr int kPP = 16;          // over-sampling rows of the sample Y
constexpr int kMaxNb = 64;
static_assert(kYWarps == kCluster, "k_yqrp: warp q pushes to cluster CTA q");

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
    pdl_wait();
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
// CTA c of the cluster holds columns [c*cn, c*cn+cn) in shared memory with
// column stride ldp (see YqrpSmem).  One step:
//   local argmax -> push the candidate (norm, index, column) to every CTA ->
//   cluster barrier -> same winner and Householder vector everywhere ->
//   update of the untaken columns, 4 lanes per column.
// Column moves for a panel from its b selections (b <= 64): selected columns
// go to the front in selection order; the displaced low positions (not
// selected), in increasing order, fill the vacated high positions (selected
// with index >= b) in increasing order.  plan_src/plan_dst hold b + (number of
// high selections) moves.  A selection outside [0, N) or a repeated one (only
// possible after non-finite values) flags status and plans no move.  Called
// by every thread of one block (a multiple of 32 threads); s_sel, in_low and
// lowpos (kMaxNb each) are shared.  Warp ballots replace the O(b^2) loops.
SKL_DEV void perm_plan_block(const int* s_sel, int* in_low, int* lowpos, int b, int N,
                             int* __restrict__ plan_src, int* __restrict__ plan_dst,
                             int* __restrict__ plan_n, unsigned* __restrict__ status)
{
    const int t = threadIdx.x, lane = t & 31, wid = t >> 5, nw = blockDim.x >> 5;
    const unsigned full = 0xffffffffu;
    // warp wid checks selections wid, wid + nw, ...: range and repeats
    bool bad = false;
    for (int tt = wid; tt < b; tt += nw) {
        const int v = s_sel[tt];
        const bool dup = (lane < tt && s_sel[lane] == v) || (lane + 32 < tt && s_sel[lane + 32] == v);
        bad = bad || __any_sync(full, dup) || v < 0 || v >= N;
    }
    if (t < kMaxNb) in_low[t] = 0;
    if (__syncthreads_or(bad)) {
        if (t == 0) {
            *plan_n = 0;
            dev_flag(status, kDevErrQrSelect);
        }
        return;
    }
    if (t < b && s_sel[t] < b) in_low[s_sel[t]] = 1;
    __syncthreads();
    if (wid == 0) {
        // displaced low positions, increasing
        int base = 0;
        for (int c = 0; c < b; c += 32) {
            const int pos = c + lane;
            const bool z = pos < b && !in_low[pos];
            const unsigned m = __ballot_sync(full, z);
            if (z) lowpos[base + __popc(m & ((1u << lane) - 1u))] = pos;
            base += __popc(m);
        }
    }
    __syncthreads();
    for (int tt = wid; tt < b; tt += nw) {
        const int hs = s_sel[tt];
        if (lane == 0) {
            plan_src[tt] = hs;
            plan_dst[tt] = tt;
        }
        if (hs >= b) {
            // rank of hs among the high selections
            const int u0 = lane < b ? s_sel[lane] : -1;
            const int u1 = lane + 32 < b ? s_sel[lane + 32] : -1;
            const int rk = __popc(__ballot_sync(full, u0 >= b && u0 < hs)) +
                           __popc(__ballot_sync(full, u1 >= b && u1 < hs));
            if (lane == 0) {
                plan_src[b + rk] = lowpos[rk];
                plan_dst[b + rk] = hs;
            }
        }
    }
    const int n_extra = __syncthreads_count(t < b && s_sel[t] >= b);
    if (t == 0) *plan_n = b + n_extra;
}

// Shared-memory budget of one CTA of the cluster kernels.
constexpr size_t kClusterSmemBudget = 200 * 1024;

// Column stride of the sample block in shared memory.  The update phase reads
// 8 columns x 4 consecutive rows per warp: a float stride of 4 x odd puts those
// 32 words in 32 distinct banks (an odd stride, conflict-free for one thread
// per column, gives 2-way conflicts there).  The padded stride is used when it
// fits the budget; FP64 keeps the odd stride.
// Warp-wide argmax of (value, index) pairs: the largest value, ties to the
// smallest index.  Index -1 marks "no candidate" and carries value -1, below
// every real value (norms, or -0.5 for a NaN norm).  Every lane returns the
// result; warp_argmax_lane also returns a lane that held it.  Generic
// types: an xor tree with that total order.
template <typename T>
SKL_DEV int warp_argmax_lane(T& v, int& i)
{
    int src = threadIdx.x & 31;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const T xv = __shfl_xor_sync(0xffffffffu, v, o);
        const int xi = __shfl_xor_sync(0xffffffffu, i, o);
        const int xs = __shfl_xor_sync(0xffffffffu, src, o);
        if (xv > v || (xv == v && xi >= 0 && (i < 0 || xi < i))) {
            v = xv;
            i = xi;
            src = xs;
        }
    }
    return src;
}
template <typename T>
SKL_DEV void warp_argmax(T& v, int& i)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const T xv = __shfl_xor_sync(0xffffffffu, v, o);
        const int xi = __shfl_xor_sync(0xffffffffu, i, o);
        if (xv > v || (xv == v && xi >= 0 && (i < 0 || xi < i))) {
            v = xv;
            i = xi;
        }
    }
}
// float: the value mapped to an unsigned key with the same order, then one
// warp max over the keys and one warp min over the indices holding the max
// (redux.sync), instead of five dependent shuffle rounds.  -0.0 does not
// occur (norms are sums of squares from +0).
SKL_DEV unsigned f32_order_key(float v)
{
    const unsigned u = __float_as_uint(v);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
SKL_DEV float f32_from_order_key(unsigned k)
{
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}
template <>
SKL_DEV int warp_argmax_lane<float>(float& v, int& i)
{
    const unsigned k = f32_order_key(v);
    const unsigned km = __reduce_max_sync(0xffffffffu, k);
    const unsigned im = __reduce_min_sync(0xffffffffu, k == km ? (unsigned)i : 0xffffffffu);
    const int src = __ffs(__ballot_sync(0xffffffffu, k == km && (unsigned)i == im)) - 1;
    v = f32_from_order_key(km);
    i = (int)im;
    return src;
}
template <>
SKL_DEV void warp_argmax<float>(float& v, int& i)
{
    const unsigned k = f32_order_key(v);
    const unsigned km = __reduce_max_sync(0xffffffffu, k);
    i = (int)__reduce_min_sync(0xffffffffu, k == km ? (unsigned)i : 0xffffffffu);
    v = f32_from_order_key(km);
}

template <typename T>
struct YqrpSmem {
    static int ldp_odd(int nbp) { return nbp | 1; }
    static int ldp_pad(int nbp)
    {
        int l = (nbp + 3) & ~3;
        if (((l >> 2) & 1) == 0) l += 4;
        return l;
    }
    static size_t bytes(int ldp, int nbp, int cn)
    {
        size_t s = (size_t)ldp * cn * sizeof(T);            // Ys
        s += (size_t)cn * sizeof(T);                        // nrm
        s += (size_t)cn + 16;                               // taken
        s = (s + 15) & ~(size_t)15;
        s += 2 * (size_t)kCluster * nbp * sizeof(T);        // all candidates' columns [2][16][nbp]
        return s + 256;
    }
    static int pick_ldp(int nbp, int cn)
    {
        if (sizeof(T) == 4 && bytes(ldp_pad(nbp), nbp, cn) <= kClusterSmemBudget) return ldp_pad(nbp);
        return ldp_odd(nbp);
    }
};

// One CTA per SM (min blocks 1): ptxas may use up to 128 registers a thread
// instead of capping the update loop at 40 with spills.
template <typename T>
__global__ void __launch_bounds__(kYThreads, 1)
k_yqrp(const T* __restrict__ Y, int ldy, int nbp, int ldp, int j0, int N, int b, int* __restrict__ sel,
       int* __restrict__ plan_src, int* __restrict__ plan_dst, int* __restrict__ plan_n,
       unsigned* __restrict__ status)
{
    pdl_wait();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const unsigned crank = cluster_ctarank();
    const int cn = (N + kCluster - 1) / kCluster;
    const int c0 = (int)crank * cn;
    const int ncols = max(0, min(cn, N - c0));
    T* Ys = (T*)smem_raw;
    T* nrm = Ys + (size_t)ldp * cn;
    unsigned char* taken = (unsigned char*)(nrm + cn);
    size_t off = ((size_t)ldp * cn * sizeof(T) + cn * sizeof(T) + cn + 16 + 15) & ~(size_t)15;
    // candidates pushed by every CTA of the cluster, double-buffered by step
    // parity: [2][16][nbp] columns, [2][16] norms and indices
    T* allc2 = (T*)(smem_raw + off);
    __shared__ T s_red_v[kYWarps];
    __shared__ int s_red_i[kYWarps];
    __shared__ T s_cv2[2][kCluster];
    __shared__ int s_ci2[2][kCluster];
    __shared__ int s_sel[kMaxNb];   // CTA 0: the selections, for the move plan
    __shared__ int s_inlow[kMaxNb];
    __shared__ int s_lowpos[kMaxNb];

    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    for (int e = tid; e < nbp * ncols; e += kYThreads) {
        int r = e % nbp, c = e / nbp;
        Ys[r + (size_t)c * ldp] = Y[r + (int64_t)(j0 + c0 + c) * ldy];
    }
    for (int c = tid; c < cn; c += kYThreads) taken[c] = (c < ncols) ? 0 : 1;
    __syncthreads();
    for (int c = tid; c < ncols; c += kYThreads) {
        const T* col = Ys + (size_t)c * ldp;
        T ss = T(0);
        for (int r = 0; r < nbp; ++r) ss += col[r] * col[r];
        nrm[c] = ss;
    }
    __syncthreads();

    // this thread's best column (largest norm; ties -> smallest index): from a
    // scan for the first step, then from the norms the update phase computes
    T bv = T(-1);
    int bi = -1;
    for (int c = tid; c < ncols; c += kYThreads) {
        // a NaN norm ranks below every real one but stays selectable, so
        // a winner always exists while untaken columns remain
        const T nv = nrm[c] == nrm[c] ? nrm[c] : T(-0.5);
        if (!taken[c] && nv > bv) { bv = nv; bi = c; }
    }
    // every CTA of the cluster has started before the first remote store
    cluster_sync();
    for (int s = 0; s < b; ++s) {
        const int p = s & 1;
        // (a) local argmax
        warp_argmax(bv, bi);
        if (lane == 0) { s_red_v[wid] = bv; s_red_i[wid] = bi; }
        __syncthreads();
        int li;   // this CTA's candidate, reduced redundantly by every warp (no second barrier)
        {
            // lanes 16-31 repeat the 16 warps' candidates (no change to the argmax)
            T ov = s_red_v[lane & (kYWarps - 1)];
            int oi = s_red_i[lane & (kYWarps - 1)];
            warp_argmax(ov, oi);
            // push this CTA's candidate to slot crank of every CTA
            if (wid == 0 && lane < kCluster) {
                dsmem_st(&s_cv2[p][crank], lane, ov);
                dsmem_st_s32(&s_ci2[p][crank], lane, (oi >= 0) ? c0 + oi : -1);
            }
            li = oi;
        }
        T* allc = allc2 + (size_t)p * kCluster * nbp;   // [16][nbp] of this step
        {
            // warp q pushes rows s.. of the candidate column to CTA q's slot crank
            T* mine = allc + (size_t)crank * nbp;
            const T* srcc = Ys + (size_t)(li >= 0 ? li : 0) * ldp;
            bool done = false;
            if constexpr (sizeof(T) == 4) {
                if (((ldp | nbp) & 3) == 0) {   // 16-byte rows: from row s rounded down to 4
                    const int r0 = s & ~3;
                    for (int r = r0 + 4 * lane; r < nbp; r += 128) {
                        const float4 v = li >= 0 ? *(const float4*)(srcc + r) : make_float4(0.f, 0.f, 0.f, 0.f);
                        dsmem_st_v4f32((float*)(mine + r), (unsigned)wid, v);
                    }
                    done = true;
                }
            }
            if (!done)
                for (int r = s + lane; r < nbp; r += 32)
                    dsmem_st(&mine[r], (unsigned)wid, (li >= 0) ? srcc[r] : T(0));
        }
        // (b) the barrier's release / acquire makes every CTA's pushes visible
        cluster_sync();
        const T* s_cv = s_cv2[p];
        const int* s_ci = s_ci2[p];
        // winner and Householder vector, in every warp (no broadcast barrier);
        // lanes 16-31 repeat the 16 candidates
        T ov = s_cv[lane & (kCluster - 1)];
        int oi = s_ci[lane & (kCluster - 1)];
        const int orank = warp_argmax_lane(ov, oi) & (kCluster - 1);
        const T* wc = allc + orank * nbp;
        T sg = T(0);
        for (int r = s + 1 + lane; r < nbp; r += 32) sg += wc[r] * wc[r];
        sg = warp_sum(sg);
        T beta, tau, scale;
        householder(wc[s], sg, beta, tau, scale);
        const int win_local = (oi >= c0 && oi < c0 + ncols) ? oi - c0 : -1;
        if (tid == 0) {
            if (crank == 0) {
                sel[s] = oi;
                s_sel[s] = oi;
            }
            if (win_local >= 0) taken[win_local] = 1;   // read again only after the next barrier
        }
        // (c) H = I - tau v v^T on the untaken local columns, new norms (rows > s):
        // 4 lanes per column, passes uniform across the CTA (quad shuffles).
        // v_s = 1 and v_r = scale * wc[r] below, so with u = sum_{r>s} wc[r] col[r]:
        // w = tau (col[s] + scale u), col[s] -= w, col[r] -= (w scale) wc[r].
        // Row s is read and written by the quad's first lane only.  Lane q4 of a
        // quad owns rows s+1+q4+4i: their wc values stay in registers for the
        // step, the column's values between the dot product and the update
        // (fully unrolled over i, with the warp-uniform chunk count nI).
        {
            constexpr int kRL = (kMaxNb + kPP + 3) / 4;   // rows below s per lane, at most
            const int q4 = tid & 3;
            const int gcol = tid >> 2;
            const int per_pass = kYThreads / 4;
            const int nI = (nbp - s + 2) >> 2;   // ceil((nbp - s - 1) / 4)
            T wv[kRL];
#pragma unroll
            for (int i = 0; i < kRL; ++i) {
                const int r = s + 1 + q4 + 4 * i;
                wv[i] = (i < nI && r < nbp) ? wc[r] : T(0);
            }
            bv = T(-1);
            bi = -1;
            for (int base = 0; base < ncols; base += per_pass) {
                const int c = base + gcol;
                const bool act = c < ncols && !taken[c] && c != win_local;
                T* col = Ys + (size_t)(act ? c : 0) * ldp;
                T yv[kRL];
                T u = T(0), cs = T(0);
                if (act && q4 == 0) cs = col[s];
#pragma unroll
                for (int i = 0; i < kRL; ++i) {
                    if (i >= nI) break;
                    const int r = s + 1 + q4 + 4 * i;
                    yv[i] = T(0);
                    if (act && r < nbp) {
                        yv[i] = col[r];
                        u += wv[i] * yv[i];
                    }
                }
                u += __shfl_xor_sync(0xffffffffu, u, 1);
                u += __shfl_xor_sync(0xffffffffu, u, 2);
                cs = __shfl_sync(0xffffffffu, cs, lane & ~3);
                const T w = tau * (cs + scale * u);
                const T ws = w * scale;
                T ss = T(0);
#pragma unroll
                for (int i = 0; i < kRL; ++i) {
                    if (i >= nI) break;
                    const int r = s + 1 + q4 + 4 * i;
                    if (act && r < nbp) {
                        const T y = yv[i] - ws * wv[i];
                        col[r] = y;
                        ss += y * y;
                    }
                }
                if (act && q4 == 0) col[s] = cs - w;
                ss += __shfl_xor_sync(0xffffffffu, ss, 1);
                ss += __shfl_xor_sync(0xffffffffu, ss, 2);
                if (act) {   // candidate for the next step (columns ascend across passes)
                    const T nv = ss == ss ? ss : T(-0.5);
                    if (nv > bv) { bv = nv; bi = c; }
                }
            }
        }
        // no barrier here: the next step's first block barrier (after each warp
        // publishes its candidate) orders these column updates before the
        // winner's column is pushed, and the candidate buffers alternate by step
    }
    __syncthreads();   // the selections written by thread 0, for the move plan
    // CTA 0 plans the panel's column moves while the cluster drains
    if (crank == 0) perm_plan_block(s_sel, s_inlow, s_lowpos, b, N, plan_src, plan_dst, plan_n, status);
    cluster_sync();   // keep shared memory alive until every CTA finished reading it
}

// ------------------------------------------- Y-QRP, registers (FP32) -----
// The same pivot selection as k_yqrp with the sample block held in registers
// instead of shared memory: the quad (4 lanes) of column slot q owns local
// columns q, q + 128, ... (NCQ of them) and lane l4 of the quad holds rows
// 2 (l4 + 4 j) and 2 (l4 + 4 j) + 1, j < 10, of each, so a column's dot
// product is a quad reduction.  Only the selections leave the kernel (the
// sample's own R is discarded), so a finished row is set to zero when its
// step ends; with rows < s zero, the step's reflector v (v_s = 1, v_r =
// scale Y(r, winner) below, zero above) makes the update y -= (tau v^T y) v
// and the next norms ||y||^2 uniform over all 20 rows, in packed FP32x2
// FMAs, with no shared-memory traffic for the block.
// Each warp's best column is staged in shared memory by its quad before the
// block barrier; after it, warp q pushes the CTA candidate's column
// (16-byte remote stores) and its norm, index, tau and scale to CTA q.
constexpr int kYRegPairsMax = 10;              // row pairs per lane: 80 rows per quad
constexpr int kYRegRows = 8 * kYRegPairsMax;   // = kMaxNb + kPP

SKL_DEV float2 ffma2(float2 a, float2 b, float2 c)
{
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rc, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "mov.b64 rc, {%6, %7};\n\tfma.rn.f32x2 rd, ra, rb, rc;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return d;
}
SKL_DEV float2 fmul2(float2 a, float2 b)
{
    float2 d;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\tmov.b64 ra, {%2, %3};\n\tmov.b64 rb, {%4, %5};\n\t"
        "mul.rn.f32x2 rd, ra, rb;\n\tmov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d.x), "=f"(d.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return d;
}
SKL_DEV float quad_sum(float x)
{
    x += __shfl_xor_sync(0xffffffffu, x, 1);
    x += __shfl_xor_sync(0xffffffffu, x, 2);
    return x;
}

// Candidate exchange, ASYNC = true: each step's pushes are st.async stores
// that complete bytes on an mbarrier of the receiving CTA (armed once per
// step with the 16 senders' bytes, alternating by step parity), so a CTA waits
// for its own incoming data instead of a cluster-wide barrier.  Every sender
// always sends its 20 granules and message (zeros without a candidate), so
// the byte count is fixed.  The wait is bounded: past the limit the kernel
// sets kStatusTcTimeout, plans no column moves and leaves the step loop.
constexpr unsigned kYWaitLimit = 1u << 22;

SKL_DEV void st_async_v4(float* local_dst, unsigned rank, float4 v, uint64_t* local_bar)
{
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.f32 [%0], {%1, %2, %3, %4}, [%5];" ::"r"(
                     dsmem_addr(local_dst, rank)),
                 "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w), "r"(dsmem_addr(local_bar, rank))
                 : "memory");
}

template <int NCQ, int NP, bool ASYNC>
__global__ void __launch_bounds__(kYThreads, 1)
k_yqrp_reg(const float* __restrict__ Y, int ldy, int nbp, int j0, int N, int b, int* __restrict__ sel,
           int* __restrict__ plan_src, int* __restrict__ plan_dst, int* __restrict__ plan_n,
           unsigned* __restrict__ status)
{
    pdl_wait();
    constexpr int kQuads = kYThreads / 4;
    constexpr int kYRegPairs = NP;                                      // row pairs per lane
    constexpr int kGran = 2 * NP;                                       // 16-byte row groups
    constexpr unsigned kYSendBytes = kGran * 16 + 16;                   // per sender and step
    __shared__ float s_wv[kYWarps];                                     // each warp's candidate
    __shared__ int s_wi[kYWarps];
    __shared__ __align__(16) float s_wstage[kYWarps][kYRegRows];       // ... and its column
    __shared__ __align__(16) float4 s_cand[2][kCluster];               // norm, index, tau
    __shared__ __align__(16) float s_col[2][kCluster][kYRegRows];      // the CTAs' candidates' v
    __shared__ __align__(8) uint64_t s_full[2];
    __shared__ int s_sel[kMaxNb];
    __shared__ int s_inlow[kMaxNb];
    __shared__ int s_lowpos[kMaxNb];

    const unsigned crank = cluster_ctarank();
    const int cn = (N + kCluster - 1) / kCluster;
    const int c0 = (int)crank * cn;
    const int ncols = max(0, min(cn, N - c0));
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int q4 = tid & 3, quad = tid >> 2;

    float2 y[NCQ][kYRegPairs];
    unsigned taken = 0;   // bit jj: slot jj taken or past the CTA's columns
#pragma unroll
    for (int jj = 0; jj < NCQ; ++jj) {
        const int lc = jj * kQuads + quad;
        const bool ok = lc < ncols;
        if (!ok) taken |= 1u << jj;
        const float* col = Y + (int64_t)(ok ? j0 + c0 + lc : j0) * ldy;
#pragma unroll
        for (int j = 0; j < kYRegPairs; ++j) {
            const int r = 2 * (q4 + 4 * j);
            y[jj][j] = (ok && r < nbp) ? *reinterpret_cast<const float2*>(col + r) : make_float2(0.f, 0.f);
        }
    }
    // this quad's best untaken column (largest norm, ties -> smallest index)
    float bv = -1.f;
    int bi = -1;
#pragma unroll
    for (int jj = 0; jj < NCQ; ++jj) {
        float2 a = make_float2(0.f, 0.f);
#pragma unroll
        for (int j = 0; j < kYRegPairs; ++j) a = ffma2(y[jj][j], y[jj][j], a);
        const float ss = quad_sum(a.x + a.y);
        const float nv = ss == ss ? ss : -0.5f;   // a NaN norm ranks below every real one
        if (!((taken >> jj) & 1u) && nv > bv) { bv = nv; bi = jj * kQuads + quad; }
    }
    if (ASYNC && tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_full[0])) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&s_full[1])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // every CTA of the cluster has started (and initialised its barriers)
    // before the first remote store
    cluster_sync();

    bool failed = false;
    for (int s = 0; s < b; ++s) {
        const int p = s & 1;
        // (a) each warp's candidate: its quad stages the column (rows < s are
        // zero); bv = ||y_{>=s}||^2 from the previous update
        warp_argmax(bv, bi);
        if (bi >= 0 && (lane >> 2) == ((bi % kQuads) & 7)) {
            const int jo = bi / kQuads;
#pragma unroll
            for (int jj = 0; jj < NCQ; ++jj) {
                if (jj != jo) continue;
#pragma unroll
                for (int j = 0; j < kYRegPairs; ++j)
                    *reinterpret_cast<float2*>(&s_wstage[wid][2 * (q4 + 4 * j)]) = y[jj][j];
            }
        }
        if (lane == 0) { s_wv[wid] = bv; s_wi[wid] = bi; }
        __syncthreads();
        if (ASYNC && tid == 0)
            asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(
                             smem_u32(&s_full[p])),
                         "r"(kYSendBytes * kCluster)
                         : "memory");
        // (b) the CTA's candidate and its reflector, from alpha = y_s and the
        // norm the argmax used, ||y_{>=s}||: beta = -sign(alpha) ||y||, tau =
        // (beta - alpha) / beta, v_s = 1, v_{>s} = y_{>s} / (alpha - beta), zero
        // above.  (Any reflector onto e_s serves: the sample's own R is
        // discarded.)  Warp q sends v and the message to CTA q of the cluster.
        float ov = s_wv[lane & (kYWarps - 1)];
        int oi = s_wi[lane & (kYWarps - 1)];
        warp_argmax(ov, oi);
        const int ow = oi >= 0 ? (oi % kQuads) >> 3 : 0;
        const float alpha = s_wstage[ow][s];
        float tau = 0.f, scale = 0.f;
        if (oi >= 0 && ov > 0.f) {
            const float nrm = ov * rsqrtf(ov);
            const float beta = alpha >= 0.f ? -nrm : nrm;
            tau = (beta - alpha) * __frcp_rn(beta);
            scale = __frcp_rn(alpha - beta);
        }
        if (lane < kGran) {
            const int r = 4 * lane;
            float4 g = *reinterpret_cast<const float4*>(&s_wstage[ow][r]);
            g.x = r > s ? scale * g.x : (r == s ? 1.f : 0.f);
            g.y = r + 1 > s ? scale * g.y : (r + 1 == s ? 1.f : 0.f);
            g.z = r + 2 > s ? scale * g.z : (r + 2 == s ? 1.f : 0.f);
            g.w = r + 3 > s ? scale * g.w : (r + 3 == s ? 1.f : 0.f);
            if (oi < 0) g = make_float4(0.f, 0.f, 0.f, 0.f);
            if constexpr (ASYNC)
                st_async_v4(&s_col[p][crank][r], (unsigned)wid, g, &s_full[p]);
            else if (oi >= 0)
                dsmem_st_v4f32(&s_col[p][crank][r], (unsigned)wid, g);
        } else if (lane == kGran) {
            const float4 msg = oi >= 0 ? make_float4(ov, __int_as_float(c0 + oi), tau, 0.f)
                                       : make_float4(-1.f, __int_as_float(-1), 0.f, 0.f);
            if constexpr (ASYNC)
                st_async_v4(reinterpret_cast<float*>(&s_cand[p][crank]), (unsigned)wid, msg, &s_full[p]);
            else
                dsmem_st_v4f32(reinterpret_cast<float*>(&s_cand[p][crank]), (unsigned)wid, msg);
        }
        // (c) every CTA's data for this step in this CTA's shared memory
        if constexpr (ASYNC) {
            const unsigned bar = smem_u32(&s_full[p]), par = (unsigned)(s >> 1) & 1u;
            unsigned done = 0;
            for (unsigned it = 0; it < kYWaitLimit && !done; ++it)
                asm volatile("{\n\t.reg .pred P;\n\tmbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 P, [%1], %2;\n\t"
                             "selp.u32 %0, 1, 0, P;\n\t}"
                             : "=r"(done)
                             : "r"(bar), "r"(par)
                             : "memory");
            if (__syncthreads_or(!done)) {
                failed = true;
                break;
            }
        } else {
            cluster_sync();
        }
        // (d) the winner and its reflector
        const float4 cm = s_cand[p][lane & (kCluster - 1)];
        float wv = cm.x;
        int wi = __float_as_int(cm.y);
        const int orank = warp_argmax_lane(wv, wi) & (kCluster - 1);
        const float wtau = s_cand[p][orank].z;
        const int win_local = (wi >= c0 && wi < c0 + ncols) ? wi - c0 : -1;
        if (tid == 0 && crank == 0) {
            sel[s] = wi;
            s_sel[s] = wi;
        }
        if (win_local >= 0 && (win_local % kQuads) == quad) taken |= 1u << (win_local / kQuads);
        const float* wc = s_col[p][orank];
        float2 v[kYRegPairs];
#pragma unroll
        for (int j = 0; j < kYRegPairs; ++j) v[j] = *reinterpret_cast<const float2*>(wc + 2 * (q4 + 4 * j));
        static_assert(kYRegPairs % 2 == 0, "row pairs are consumed two at a time");
        // (e) w = tau v^T y per slot (independent chains, interleaved)
        float w[NCQ];
#pragma unroll
        for (int jj = 0; jj < NCQ; ++jj) {
            float2 a0 = make_float2(0.f, 0.f), a1 = make_float2(0.f, 0.f);
#pragma unroll
            for (int j = 0; j < kYRegPairs; j += 2) {
                a0 = ffma2(v[j], y[jj][j], a0);
                a1 = ffma2(v[j + 1], y[jj][j + 1], a1);
            }
            w[jj] = (a0.x + a0.y) + (a1.x + a1.y);
        }
#pragma unroll
        for (int jj = 0; jj < NCQ; ++jj) w[jj] = wtau * quad_sum(w[jj]);
        // row s leaves the sample: zero it in y and in v (the lane holding row
        // s, pair s / 8), so y -= w v keeps it zero and the norms need no mask
        if (q4 == ((s >> 1) & 3)) {
            const int js = s >> 3;
            const float2 keep = (s & 1) ? make_float2(1.f, 0.f) : make_float2(0.f, 1.f);
#pragma unroll
            for (int j = 0; j < kYRegPairs; ++j) {
                if (j != js) continue;
                v[j] = fmul2(v[j], keep);
#pragma unroll
                for (int jj = 0; jj < NCQ; ++jj) y[jj][j] = fmul2(y[jj][j], keep);
            }
        }
        // y -= w v and the next norms ||y_{>s}||^2; taken slots update too
        // (their values are never read again)
        float ss[NCQ];
#pragma unroll
        for (int jj = 0; jj < NCQ; ++jj) {
            const float2 nw = make_float2(-w[jj], -w[jj]);
            float2 q0 = make_float2(0.f, 0.f), q1 = make_float2(0.f, 0.f);
#pragma unroll
            for (int j = 0; j < kYRegPairs; j += 2) {
                y[jj][j] = ffma2(nw, v[j], y[jj][j]);
                y[jj][j + 1] = ffma2(nw, v[j + 1], y[jj][j + 1]);
                q0 = ffma2(y[jj][j], y[jj][j], q0);
                q1 = ffma2(y[jj][j + 1], y[jj][j + 1], q1);
            }
            ss[jj] = (q0.x + q0.y) + (q1.x + q1.y);
        }
        bv = -1.f;
        bi = -1;
#pragma unroll
        for (int jj = 0; jj < NCQ; ++jj) {   // columns ascend with jj
            const float sq = quad_sum(ss[jj]);
            const float nv = sq == sq ? sq : -0.5f;
            if (!((taken >> jj) & 1u) && nv > bv) { bv = nv; bi = jj * kQuads + quad; }
        }
        // no barrier here: the next step's block barrier orders the staging
        // buffer's reuse, and the candidate buffers alternate by step
    }
    __syncthreads();   // the selections written by thread 0, for the move plan
    if (failed) {
        if (tid == 0) {
            atomicOr(status, kStatusTcTimeout);
            if (crank == 0) *plan_n = 0;
        }
    } else if (crank == 0) {
        perm_plan_block(s_sel, s_inlow, s_lowpos, b, N, plan_src, plan_dst, plan_n, status);
    }
    cluster_sync();   // keep shared memory alive until every CTA finished reading it
}

// -------------------------------------------------- column permutation --
// Moves the selected columns (sel, relative to j0) to positions j0..j0+b-1;
// the columns they displace fill the vacated positions in increasing order.
// plan: src[t] for t in [0, 2b): dest position dst[t] (relative) <- src.
// Planned column moves of A (rows m, ld), the sample Y (nbp rows, ldy) and
// jpvt: gather every source column into scratch, then (next launch, after all
// gathers) write them to their destinations.  Grid (x over rows of A, one y
// per planned move); the x == 0 blocks also move Y's column and jpvt.
template <typename T>
__global__ void k_perm_gather(const T* __restrict__ A, int64_t ld, int m, const T* __restrict__ Y,
                              int ldy, int nbp, const int* __restrict__ jpvt, int j0,
                              const int* __restrict__ plan_src, const int* __restrict__ plan_n,
                              T* __restrict__ tmpA, T* __restrict__ tmpY, int* __restrict__ tmpI)
{
    pdl_wait();
    const int q = blockIdx.y;
    if (q >= *plan_n) return;
    const int64_t c = j0 + plan_src[q];
    const T* src = A + c * ld;
    T* dst = tmpA + (int64_t)q * m;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x)
        dst[r] = src[r];
    if (blockIdx.x == 0) {
        for (int r = threadIdx.x; r < nbp; r += blockDim.x) tmpY[q * nbp + r] = Y[c * ldy + r];
        if (threadIdx.x == 0) tmpI[q] = jpvt[c];
    }
}

template <typename T>
__global__ void k_perm_scatter(T* __restrict__ A, int64_t ld, int m, T* __restrict__ Y, int ldy,
                               int nbp, int* __restrict__ jpvt, int j0,
                               const int* __restrict__ plan_dst, const int* __restrict__ plan_n,
                               const T* __restrict__ tmpA, const T* __restrict__ tmpY,
                               const int* __restrict__ tmpI)
{
    pdl_wait();
    const int q = blockIdx.y;
    if (q >= *plan_n) return;
    const int64_t c = j0 + plan_dst[q];
    T* dst = A + c * ld;
    const T* src = tmpA + (int64_t)q * m;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < m; r += gridDim.x * blockDim.x)
        dst[r] = src[r];
    if (blockIdx.x == 0) {
        for (int r = threadIdx.x; r < nbp; r += blockDim.x) Y[c * ldy + r] = tmpY[q * nbp + r];
        if (threadIdx.x == 0) jpvt[c] = tmpI[q];
    }
}

// ------------------------------------------------------------- panel ----
// Pivoted Householder QR of the panel P = A(j0:m, j0:j0+b) held in the
// cluster's shared memory: CTA c owns panel rows [c*R, c*R+R) (R a multiple
// of 4, rows past the panel end are zero).  Per column step s:
//   (A) cluster barrier, one batched DSMEM round trip gathers the column
//       norms below row s and the owner's row s  ->  pivot, Householder v;
//   local swap + scaling of column s;
//   dots d_c = sum_{r>=s} v_r P[r][c] for every column c != s: for c > s this
//       is w = V^T P (the rank-1 update), for c < s it is V(:,c)^T v_s, the
//       column of V^T V that the T factor needs (dlarft recurrence), so T is
//       built step by step without a separate Gram pass;
//   (B) cluster barrier, one DSMEM round trip gathers the dots;
//   update of the columns c > s and their next norms.
// Row loops use float4 (double2) vectors along the rows of a column.
template <typename T>
size_t panel_smem_bytes(int R, int b)
{
    size_t s = (size_t)R * b * sizeof(T);       // Ps
    s += 6 * (size_t)kMaxNb * sizeof(T);        // red1, red2, rowS, nrm2, rowL, dots
    s += (size_t)kMaxNb * kMaxNb * sizeof(T);   // T factor
    s += 2 * (size_t)kMaxNb * sizeof(int);      // piv history, permutation
    return s + 512;
}

template <typename T> struct Vec4T;
template <> struct Vec4T<float> { using type = float4; static constexpr int n = 4; };
template <> struct Vec4T<double> { using type = double2; static constexpr int n = 2; };

template <typename T>
SKL_DEV void v_fma(typename Vec4T<T>::type& x, T a, typename Vec4T<T>::type y);
template <>
SKL_DEV void v_fma<float>(float4& x, float a, float4 y)
{ x.x = fmaf(a, y.x, x.x); x.y = fmaf(a, y.y, x.y); x.z = fmaf(a, y.z, x.z); x.w = fmaf(a, y.w, x.w); }
template <>
SKL_DEV void v_fma<double>(double2& x, double a, double2 y)
{ x.x = fma(a, y.x, x.x); x.y = fma(a, y.y, x.y); }

template <typename T>
SKL_DEV T v_dot(typename Vec4T<T>::type a, typename Vec4T<T>::type b);
template <>
SKL_DEV float v_dot<float>(float4 a, float4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
template <>
SKL_DEV double v_dot<double>(double2 a, double2 b) { return a.x * b.x + a.y * b.y; }

// element e of a vector
template <typename T>
SKL_DEV T v_get(const typename Vec4T<T>::type& a, int e);
template <>
SKL_DEV float v_get<float>(const float4& a, int e) { return e == 0 ? a.x : e == 1 ? a.y : e == 2 ? a.z : a.w; }
template <>
SKL_DEV double v_get<double>(const double2& a, int e) { return e == 0 ? a.x : a.y; }

template <typename T>
__global__ void __launch_bounds__(kQrThreads)
k_panel(T* __restrict__ A, int64_t ld, int j0, int M, int b, int R, T* __restrict__ tau_out,
        T* __restrict__ Tout, int ldt, T* __restrict__ V, int64_t ldv, int* __restrict__ jpvt,
        T* __restrict__ Y, int ldy, int nbp, int pivot_panel, const int* __restrict__ chol_fail)
{
    pdl_wait();
    // runs only when the CholeskyQR2 panel (if any) declined this panel
    if (chol_fail && *chol_fail == 0) return;
    using V4 = typename Vec4T<T>::type;
    constexpr int VN = Vec4T<T>::n;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const unsigned crank = cluster_ctarank();
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int r0 = (int)crank * R;                      // first panel row owned
    const int nr = max(0, min(R, M - r0));              // real rows owned (rest are zero)
    T* Ps = (T*)smem_raw;                               // [b][R] column-major
    T* red1 = Ps + (size_t)R * b;
    T* red2 = red1 + kMaxNb;
    T* rowS = red2 + kMaxNb;
    T* nrm2 = rowS + kMaxNb;
    T* rowL = nrm2 + kMaxNb;
    T* dots = rowL + kMaxNb;
    T* Tl = dots + kMaxNb;                              // [b][kMaxNb], column i at Tl[i*kMaxNb]
    int* pivh = (int*)(Tl + kMaxNb * kMaxNb);
    int* perm = pivh + kMaxNb;
    __shared__ T s_beta, s_tau, s_scale;
    __shared__ int s_piv;
    const int nv = R / VN;                              // vectors per column

    // load the panel rows (zero padding past the panel end)
    for (int e = tid; e < R * b; e += kQrThreads) {
        int lr = e % R, c = e / R;
        Ps[lr + (size_t)c * R] = (lr < nr) ? A[(int64_t)(j0 + r0 + lr) + (int64_t)(j0 + c) * ld] : T(0);
    }
    __syncthreads();
    // initial partial norms over rows > 0 and row 0 values
    for (int c = wid; c < b; c += kQrWarps) {
        T ss = T(0);
        for (int lr = lane; lr < nr; lr += 32) {
            T x = Ps[lr + (size_t)c * R];
            if (r0 + lr > 0) ss += x * x;
            else rowS[c] = x;
        }
        ss = warp_sum(ss);
        if (lane == 0) red1[c] = ss;
    }
    const int steps = min(b, M);
    for (int s = 0; s < steps; ++s) {
        const unsigned own = (unsigned)(s / R);
        cluster_sync();                                  // (A) red1, rowS published
        {
            const int q = tid & 15;
#pragma unroll
            for (int pass = 0; pass < 2; ++pass) {
                const int c = s + pass * (kQrThreads / 16) + (tid >> 4);
                T x = T(0);
                if (c < b) x = dsmem_ld(&red1[c], q);
#pragma unroll
                for (int o = 8; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
                if (q == 0 && c < b) nrm2[c] = x;
            }
            if (tid < b - s) rowL[s + tid] = dsmem_ld(&rowS[s + tid], own);
        }
        __syncthreads();
        if (wid == 0) {
            int piv = s;
            T best = T(-1);
            for (int c = s + lane; c < b; c += 32) {
                T v2 = nrm2[c] + rowL[c] * rowL[c];
                if (v2 > best) { best = v2; piv = c; }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                T ob = __shfl_xor_sync(0xffffffffu, best, o);
                int op = __shfl_xor_sync(0xffffffffu, piv, o);
                if (ob > best || (ob == best && op < piv)) { best = ob; piv = op; }
            }
            if (!pivot_panel) piv = s;
            if (lane == 0) {
                T beta, tau, scale;
                householder(rowL[piv], nrm2[piv], beta, tau, scale);
                s_piv = piv;
                s_beta = beta;
                s_tau = tau;
                s_scale = scale;
                pivh[s] = piv;
            }
        }
        __syncthreads();
        const int piv = s_piv;
        const T tau = s_tau, scale = s_scale, beta = s_beta;
        for (int lr = tid; lr < R; lr += kQrThreads) {
            T a = Ps[lr + (size_t)s * R];
            if (piv != s) {
                T c = Ps[lr + (size_t)piv * R];
                Ps[lr + (size_t)piv * R] = a;
                a = c;
            }
            const int g = r0 + lr;
            if (g > s) a *= scale;
            else if (g == s) a = beta;
            Ps[lr + (size_t)s * R] = a;
        }
        __syncthreads();
        // v restricted to rows >= s: vectors of VN rows; the vector holding
        // row s gets v_s = 1 and zeros above
        const int lr_s = max(0, s - r0);
        const int q0 = lr_s / VN;
        auto vload = [&](int qv) -> V4 {
            V4 vv = reinterpret_cast<const V4*>(Ps + (size_t)s * R)[qv];
            const int base = r0 + qv * VN;
            if (base + VN - 1 >= s && base <= s) {
                T* pv = reinterpret_cast<T*>(&vv);
#pragma unroll
                for (int e = 0; e < VN; ++e) {
                    int g = base + e;
                    pv[e] = (g < s) ? T(0) : (g == s ? T(1) : pv[e]);
                }
            }
            return vv;
        };
        // dots for all columns c != s (4 per warp, covering 64 columns)
        {
            T acc[4] = {T(0), T(0), T(0), T(0)};
            for (int qv = q0 + lane; qv < nv; qv += 32) {
                const V4 vv = vload(qv);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int c = wid + q * kQrWarps;
                    if (c < b && c != s) acc[q] += v_dot<T>(vv, reinterpret_cast<const V4*>(Ps + (size_t)c * R)[qv]);
                }
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int c = wid + q * kQrWarps;
                T x = warp_sum(acc[q]);
                if (lane == 0 && c < b) red2[c] = x;
            }
        }
        cluster_sync();                                  // (B) red2 published
        {
            const int q = tid & 15;
#pragma unroll
            for (int pass = 0; pass < 2; ++pass) {
                const int c = pass * (kQrThreads / 16) + (tid >> 4);
                T x = T(0);
                if (c < b) x = dsmem_ld(&red2[c], q);
#pragma unroll
                for (int o = 8; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
                if (q == 0 && c < b) dots[c] = x;
            }
        }
        __syncthreads();
        // T(0:s, s) = -tau * T(0:s, 0:s) * (V(:,0:s)^T v_s), T(s,s) = tau
        if (wid == 1) {
            for (int i = lane; i < s; i += 32) {
                T acc = T(0);
                for (int c = i; c < s; ++c) acc += Tl[i + c * kMaxNb] * dots[c];
                Tl[i + s * kMaxNb] = -tau * acc;
            }
            if (lane == 0) Tl[s + s * kMaxNb] = tau;
        }
        // update columns c > s, next partial norms (rows > s+1) and row s+1
        {
            T ss[4] = {T(0), T(0), T(0), T(0)};
            T wq[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int c = wid + q * kQrWarps;
                wq[q] = (c < b && c > s) ? dots[c] * tau : T(0);
            }
            for (int qv = q0 + lane; qv < nv; qv += 32) {
                const V4 vv = vload(qv);
                const int base = r0 + qv * VN;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int c = wid + q * kQrWarps;
                    if (c < b && c > s) {
                        V4* pc = reinterpret_cast<V4*>(Ps + (size_t)c * R) + qv;
                        V4 x = *pc;
                        v_fma<T>(x, -wq[q], vv);
                        *pc = x;
                        const T* px = reinterpret_cast<const T*>(&x);
#pragma unroll
                        for (int e = 0; e < VN; ++e) {
                            const int g = base + e;
                            if (g > s + 1) ss[q] += px[e] * px[e];
                            else if (g == s + 1) rowS[c] = px[e];
                        }
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int c = wid + q * kQrWarps;
                T x = warp_sum(ss[q]);
                if (lane == 0 && c < b && c > s) red1[c] = x;
            }
        }
        if (tid == 0 && crank == 0) tau_out[j0 + s] = tau;
        __syncthreads();
    }
    // final permutation of the panel's columns (composition of the swaps)
    if (tid == 0) {
        for (int t = 0; t < b; ++t) perm[t] = t;
        for (int s2 = 0; s2 < steps; ++s2) {
            int p2 = pivh[s2];
            int x = perm[s2];
            perm[s2] = perm[p2];
            perm[p2] = x;
        }
    }
    if (crank == 0) {
        for (int e = tid; e < b * b; e += kQrThreads) {
            int a = e % b, c = e / b;
            Tout[a + (int64_t)c * ldt] = (a <= c) ? Tl[a + c * kMaxNb] : T(0);
        }
    }
    cluster_sync();   // no CTA leaves while others may still read its shared memory
    // write back panel: R (upper) + V (below) into A; explicit V into the V buffer
    for (int e = tid; e < nr * b; e += kQrThreads) {
        int lr = e % nr, c = e / nr;
        int g = r0 + lr;
        T x = Ps[lr + (size_t)c * R];
        A[(int64_t)(j0 + g) + (int64_t)(j0 + c) * ld] = x;
        V[(int64_t)g + (int64_t)c * ldv] = (g > c) ? x : (g == c ? T(1) : T(0));
    }
    // permute the columns j0..j0+b of the rows above the panel, of Y and of
    // jpvt: each row gathers its b values once (independent loads), then stores
    const int nabove = j0;
    for (int row = (int)crank * kQrThreads + tid; row < nabove + nbp + 1;
         row += kCluster * kQrThreads) {
        if (row < nabove || (row < nabove + nbp && Y)) {
            T* base = row < nabove ? A + row : Y + (row - nabove);
            const int64_t stride = row < nabove ? ld : (int64_t)ldy;
            T vals[kMaxNb];
#pragma unroll 8
            for (int t = 0; t < b; ++t) vals[t] = base[(int64_t)(j0 + perm[t]) * stride];
#pragma unroll 8
            for (int t = 0; t < b; ++t) base[(int64_t)(j0 + t) * stride] = vals[t];
        } else if (row == nabove + nbp) {
            int vals[kMaxNb];
            for (int t = 0; t < b; ++t) vals[t] = jpvt[j0 + perm[t]];
            for (int t = 0; t < b; ++t) jpvt[j0 + t] = vals[t];
        }
    }
}


// --------------------------------------------------- CholeskyQR2 panel ----
// Unpivoted QR of the panel P = A(j0:m, j0:j0+b) (column order from the
// sample QRP) by CholeskyQR2, then Householder reconstruction by the
// modified LU of Ballard, Demmel, Grigori, Jacquelin, Knight and Nguyen
// ("Reconstructing Householder vectors from TSQR", 2015):
//   G1 = P^T P = R1^T R1,  Q = P R1^{-1},  G2 = Q^T Q = R2^T R2,
//   Q1 = Q(0:b,:) R2^{-1},  Q1 - S = L U (no pivoting, S_kk = -sign of pivot),
//   V = [L; Q(b:,:) W],  W = R2^{-1} U^{-1},  T = -U S L^{-T},  R_H = S R2 R1,
// so I - V T V^T has Q S as its first b columns and the trailing update and
// the sample downdate use (V, T) exactly as with the column-by-column panel.
//
// The tall products (the two Grams, P R1^{-1}, Q W) are GEMMs over the whole
// GPU, the panel staying in L2; the b x b algebra runs in one CTA
// (k_chol_small1/2) with room for the registers its factorizations need:
// two warps hold the matrix a column per thread and take one 64-thread
// barrier per step; products use register-tiled block multiplies.
//
// A Cholesky pivot below 32 eps of its column's mass, or a second Gram
// farther than 1/2 from the identity (Gershgorin), means kappa(P) is too large
// for CholeskyQR2: *fail = 1, A is left untouched and the pivoted panel kernel
// launched next factors the panel instead.
// ------------------------------------------------- Q^T c for one panel --
// c(j0:m) <- (I - V T^T V^T) c(j0:m), FP64 accumulation.  w = V^T c: one
// block per column of V; the update: one warp per 32 rows, z = T^T w in smem.
template <typename T>
__global__ void k_qt_w(const T* __restrict__ V, int64_t ldv, int M, int b,
                       const double* __restrict__ c, double* __restrict__ w)
{
    pdl_wait();
    __shared__ double red[32];
    const int a = blockIdx.x;
    const T* va = V + (int64_t)a * ldv;
    double acc = 0.0;
    for (int r = a + threadIdx.x; r < M; r += blockDim.x) acc = fma((double)va[r], c[r], acc);
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) w[a] = acc;
}

template <typename T>
__global__ void k_qt_update(const T* __restrict__ V, int64_t ldv, int M, int b,
                            const T* __restrict__ Tm, int ldt, const double* __restrict__ w,
                            double* __restrict__ c)
{
    pdl_wait();
    __shared__ double z[kMaxNb];
    if (threadIdx.x < b) {
        const int i = threadIdx.x;
        double acc = 0.0;
        for (int a = 0; a <= i; ++a) acc = fma((double)Tm[a + (int64_t)i * ldt], w[a], acc);
        z[i] = acc;
    }
    __syncthreads();
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < M; r += gridDim.x * blockDim.x) {
        double acc = 0.0;
        const int amax = min(b, r + 1);   // V is zero above its diagonal
        for (int a = 0; a < amax; ++a) acc = fma((double)V[r + (int64_t)a * ldv], z[a], acc);
        c[r] -= acc;
    }
}

template <typename T>
__global__ void k_copy_block(const T* __restrict__ src, int64_t lds, T* __restrict__ dst,
                             int64_t ldd, int rows, int cols)
{
    pdl_wait();
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < rows * cols; e += gridDim.x * blockDim.x) {
        int r = e % rows, c = e / rows;
        dst[r + (int64_t)c * ldd] = src[r + (int64_t)c * lds];
    }
}

__global__ void k_iota_int(int* v, int n)
{
    pdl_wait();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = i;
}

// ------------------------------------------------------------ host side --
// Panel method: CholeskyQR2 + Householder reconstruction by default on the
// FP32 path (its tall products run at full-GPU GEMM speed), the column-by-
// column pivoted panel on the FP64 path (there the FP64 GEMMs cost more than
// the latency the pivoted panel spends); SKILLS_QR_PANEL=chol|pivoted overrides.
template <typename T>
static bool qr_chol_enabled()
{
    static const int v = [] {
        const char* e = getenv("SKILLS_QR_PANEL");
        if (e && std::string(e) == "pivoted") return 0;
        if (e && std::string(e) == "chol") return 1;
        return 2;
    }();
    if (v == 2) return std::is_same<T, float>::value;
    return v == 1;
}

struct QrPlan {
    int nb, nbp, R;
};

// nb_cap > 0 caps the panel width (a tuning choice, multiple of 8).
template <typename T>
static QrPlan qr_plan(int64_t m, int64_t d, int nb_cap = 0)
{
    QrPlan p;
    p.R = (int)((m + kCluster - 1) / kCluster);
    p.R = (p.R + 3) / 4 * 4;   // whole float4 / double2 row vectors
    int nb = (nb_cap >= 8 && nb_cap < kMaxNb) ? nb_cap / 8 * 8 : kMaxNb;
    const size_t budget = kClusterSmemBudget;
    while (nb > 8 && panel_smem_bytes<T>(p.R, nb) > budget) nb -= 8;
    if (panel_smem_bytes<T>(p.R, nb) > budget)
        fail(SKL_ERR_INVALID, "cpqr: sketch has too many rows for the shared-memory panel (m=" +
                                  std::to_string(m) + ")");
    p.nb = nb;
    p.nbp = nb + kPP;
    int64_t cn = (d + kCluster - 1) / kCluster;
    if (YqrpSmem<T>::bytes(YqrpSmem<T>::ldp_odd(p.nbp), p.nbp, (int)cn) > budget)
        fail(SKL_ERR_INVALID, "cpqr: too many columns for the shared-memory sample QRP (d=" +
                                  std::to_string(d) + ")");
    return p;
}

template <typename T>
struct QrBuffers {
    T *G, *Y, *V, *Tm, *W, *Z, *GU, *GUT, *Bm, *part, *part2, *tmp;
    int *sel, *plan_src, *plan_dst, *plan_n, *chol_fail;
    T* tmpY;      // 2 nb sample columns being moved
    int* tmpI;    // 2 nb pivot indices being moved
    T *cg, *cr1, *cx1, *cw;   // CholeskyQR2 panel: Gram, R1, R1^{-1}, R2^{-1} U^{-1}
    double *qw;
    float* tcs;   // tensor-core W = V^T A: split V and split-K partials (FP32 path)
    size_t tcs_floats;
    float* tcu;   // tensor-core A -= V Z: split V and Z (FP32 path)
    int64_t part_cap, part2_cap, tmp_rows;   // part2: split-K partials of the side stream
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
    B.part2_cap = (int64_t)kSplitMax * p.nbp * p.nb;
    B.part2 = (T*)take((size_t)B.part2_cap * sizeof(T));
    B.tmp_rows = m > p.nbp ? m : p.nbp;
    B.tmp = (T*)take((size_t)B.tmp_rows * 2 * p.nb * sizeof(T));
    B.tmpY = (T*)take((size_t)p.nbp * 2 * p.nb * sizeof(T));
    B.tmpI = (int*)take(2 * kMaxNb * sizeof(int));
    B.sel = (int*)take(kMaxNb * sizeof(int));
    B.plan_src = (int*)take(2 * kMaxNb * sizeof(int));
    B.plan_dst = (int*)take(2 * kMaxNb * sizeof(int));
    B.plan_n = (int*)take(sizeof(int));
    B.chol_fail = (int*)take(sizeof(int));
    B.cg = (T*)take((size_t)p.nb * p.nb * sizeof(T));
    B.cr1 = (T*)take((size_t)p.nb * p.nb * sizeof(T));
    B.cx1 = (T*)take((size_t)p.nb * p.nb * sizeof(T));
    B.cw = (T*)take((size_t)p.nb * p.nb * sizeof(T));
    B.qw = (double*)take(kMaxNb * sizeof(double));
    B.tcs_floats = std::is_same<T, float>::value ? tc_vta_scratch_floats(m) : 0;
    B.tcs = (float*)take(B.tcs_floats * sizeof(float));
    B.tcu = (float*)take((std::is_same<T, float>::value ? tc_update_scratch_floats(m, d) : 0) *
                         sizeof(float));
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
    allow_max_dynamic_smem(fn);
    (void)smem;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kCluster, 1, 1);
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[2];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = kCluster;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;   // see launch.cuh
    at[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl_enabled() ? 2 : 1;
    SKL_CUDA(cudaLaunchKernelExC(&cfg, fn, args));
    SKL_LAUNCHED();
}

// Launch shape of the register sample QRP for nbp sample rows and N columns:
// row pairs per lane np (8: nbp <= 64, 10: nbp <= 80) and column slots per
// quad ncq (at most 3 with 10 pairs, 5 with 8: what 128 registers a thread
// hold), or ncq = 0 for the shared-memory kernel (FP64, wider samples).
// SKILLS_YQRP_REG=0 keeps the latter.
struct YRegShape {
    int ncq, np;
};
template <typename T>
static YRegShape yqrp_reg_shape(int nbp, int N)
{
    static const bool off = [] {
        const char* e = getenv("SKILLS_YQRP_REG");
        return e && e[0] == '0';
    }();
    if (!std::is_same<T, float>::value || off || nbp > kYRegRows || (nbp & 1)) return {0, 0};
    const int np = nbp <= 64 ? 8 : 10;
    const int cn = (N + kCluster - 1) / kCluster;
    const int ncq = std::max(1, (cn + kYThreads / 4 - 1) / (kYThreads / 4));
    return {ncq <= (np == 8 ? 5 : 3) ? ncq : 0, np};
}

// The register sample QRP's exchange: mbarrier-completed remote stores
// (default) or remote stores plus a cluster barrier (SKILLS_YQRP_ASYNC=0).
static bool yqrp_async()
{
    static const bool v = [] {
        const char* e = getenv("SKILLS_YQRP_ASYNC");
        return !(e && e[0] == '0');
    }();
    return v;
}

static const void* yqrp_reg_kernel(YRegShape sh, bool async)
{
#define YREG(C, P) (async ? (const void*)k_yqrp_reg<C, P, true> : (const void*)k_yqrp_reg<C, P, false>)
    if (sh.np == 8) {
        switch (sh.ncq) {
        case 1: return YREG(1, 8);
        case 2: return YREG(2, 8);
        case 3: return YREG(3, 8);
        case 4: return YREG(4, 8);
        default: return YREG(5, 8);
        }
    }
    switch (sh.ncq) {
    case 1: return YREG(1, 10);
    case 2: return YREG(2, 10);
    default: return YREG(3, 10);
    }
#undef YREG
}

// Event pairs around QR sub-steps (profiling only).
struct QrTimer {
    double* acc;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> marks;
    std::vector<cudaEvent_t> pool;
    size_t used = 0;
    cudaStream_t st;
    cudaEvent_t get()
    {
        if (used == pool.size()) {
            cudaEvent_t e;
            SKL_CUDA(cudaEventCreate(&e));
            pool.push_back(e);
        }
        return pool[used++];
    }
    cudaEvent_t begin()
    {
        if (!acc) return nullptr;
        cudaEvent_t e = get();
        SKL_CUDA(cudaEventRecord(e, st));
        return e;
    }
    void end(int slot, cudaEvent_t b)
    {
        if (!acc) return;
        cudaEvent_t e = get();
        SKL_CUDA(cudaEventRecord(e, st));
        marks.push_back({slot, {b, e}});
    }
    void finish()
    {
        if (!acc) return;
        SKL_CUDA(cudaStreamSynchronize(st));
        for (auto& mk : marks) {
            float ms = 0.f;
            SKL_CUDA(cudaEventElapsedTime(&ms, mk.second.first, mk.second.second));
            acc[mk.first] += ms;
        }
        for (auto e : pool) cudaEventDestroy(e);
    }
};

template <typename T>
static void qr_core(T* A, int64_t m, int64_t d, int64_t ld, int* jpvt, T* tau, void* work,
                    unsigned* status, cudaStream_t st, double* c, bool pivoting, double* qr_prof,
                    int nb_cap)
{
    QrTimer tm{qr_prof, {}, {}, 0, st};
    QrPlan p = qr_plan<T>(m, d, nb_cap);
    QrBuffers<T> B = qr_carve<T>(work, m, d, p, nullptr);
    const int nb = p.nb, nbp = p.nbp;
    const int64_t mn = m < d ? m : d;
    launch_k(k_iota_int, (unsigned)((d + 255) / 256), 256, 0, st, jpvt, (int)d);
    SKL_LAUNCHED();
    if (pivoting) {
        int64_t cnt = (int64_t)nbp * m;
        launch_k(k_gaussian<T>, (unsigned)((cnt + 255) / 256 < 2048 ? (cnt + 255) / 256 : 2048), 256, 0, st, 
            B.G, cnt, 0x5eed000000000012ull);
        SKL_LAUNCHED();
        cudaEvent_t t0 = tm.begin();
        gemm<T>(false, false, nbp, (int)d, (int)m, T(1), B.G, nbp, A, ld, T(0), B.Y, nbp, B.part,
                B.part_cap, st);
        tm.end(8, t0);
    }
    // one sample-block stride for every launch of this factorisation, chosen
    // at the largest column count (later launches need no more shared memory)
    const int ycn_max = (int)((d + kCluster - 1) / kCluster);
    const int yldp = YqrpSmem<T>::pick_ldp(nbp, ycn_max);
    const size_t ysm_max = YqrpSmem<T>::bytes(yldp, nbp, ycn_max);
    const size_t psm = panel_smem_bytes<T>(p.R, nb);

    // CholeskyQR2 panels, not the last panel (it has no sample QRP ordering),
    // rows 0..b-1 of a panel inside CTA 0.  Unpivoted factorisations (the
    // full-rank noCPQR and Blendenpik sketches) use them too: a panel whose
    // Cholesky breaks down or whose second Gram strays from the identity
    // falls back to the Householder panel (chol_fail)
    const bool use_chol = nb <= 64 && std::is_same<T, float>::value && qr_chol_enabled<T>();

    // Two streams.  The sample work of panel j (Y downdate, the sample QRP of
    // panel j+1) needs only V, T and R12 = A12 - V1 Z, so it runs on a
    // high-priority side stream: the part that needs V and T alone (GU, GUT, B
    // and G -= GUT V^T) overlaps W and R12, the rest (Y2 -= B R12, the next
    // sample QRP) overlaps the big trailing update and Q^T c; panel j+1's
    // permutation waits for the side stream's events.  (R12 is the first b
    // rows of the trailing update, done ahead of the other rows.)
    cudaStream_t side = nullptr;
    cudaEvent_t evV = nullptr, evR = nullptr, evY = nullptr, evG = nullptr, evD = nullptr;
    if (pivoting) {
        int lo = 0, hi = 0;
        SKL_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        SKL_CUDA(cudaStreamCreateWithPriority(&side, cudaStreamNonBlocking, hi));
        SKL_CUDA(cudaEventCreateWithFlags(&evV, cudaEventDisableTiming));
        SKL_CUDA(cudaEventCreateWithFlags(&evR, cudaEventDisableTiming));
        SKL_CUDA(cudaEventCreateWithFlags(&evY, cudaEventDisableTiming));
        SKL_CUDA(cudaEventCreateWithFlags(&evG, cudaEventDisableTiming));
        SKL_CUDA(cudaEventCreateWithFlags(&evD, cudaEventDisableTiming));
    }
    struct StreamGuard {
        cudaStream_t s;
        cudaEvent_t ev[5];
        ~StreamGuard()
        {
            for (cudaEvent_t e : ev)
                if (e) cudaEventDestroy(e);
            if (s) cudaStreamDestroy(s);
        }
    } guard{side, {evV, evR, evY, evG, evD}};
    QrTimer tms{qr_prof, {}, {}, 0, side};
    bool side_pending = false;

    auto launch_yqrp = [&](int64_t j, int b, int N, cudaStream_t s, QrTimer& t) {
        int jj = (int)j;
        int ldy = nbp;
        const T* Yc = B.Y;
        int* sel = B.sel;
        int nbv = nbp;
        int ldpv = yldp;
        int* psrc = B.plan_src;
        int* pdst = B.plan_dst;
        int* pn = B.plan_n;
        unsigned* stp = status;
        void* args[] = {(void*)&Yc, &ldy, (void*)&nbv, &ldpv, &jj, (void*)&N, (void*)&b, &sel, &psrc,
                        &pdst, &pn, &stp};
        cudaEvent_t t0 = t.begin();
        const YRegShape sh = yqrp_reg_shape<T>(nbp, N);
        if (sh.ncq > 0) {
            void* rargs[] = {(void*)&Yc, &ldy, (void*)&nbv, &jj, (void*)&N, (void*)&b, &sel, &psrc,
                             &pdst, &pn, &stp};
            launch_cluster<T>(yqrp_reg_kernel(sh, yqrp_async()), dim3(kYThreads), 0, s, rargs);
        } else {
            launch_cluster<T>((const void*)k_yqrp<T>, dim3(kYThreads), ysm_max, s, args);
        }
        t.end(0, t0);
    };

    for (int64_t j = 0; j < mn; j += nb) {
        const int b = (int)std::min<int64_t>(nb, std::min<int64_t>(d - j, m - j));
        const bool last = (j + nb >= m) || (j + nb >= d);
        const int M = (int)(m - j);
        const int N = (int)(d - j);
        trace_phase(st, "qr: panel start");
        if (side_pending) {
            // the sample QRP of this panel (evY) before the permutation; the
            // side stream's last use of V (evG) before the panel rewrites it
            SKL_CUDA(cudaStreamWaitEvent(st, evY, 0));
        }
        if (pivoting && !last) {
            int jj = (int)j;
            if (j == 0) launch_yqrp(j, b, N, st, tm);
            trace_phase(st, "qr: yqrp");
            cudaEvent_t t0 = tm.begin();
            // the sample QRP planned the moves (plan_src/plan_dst/plan_n)
            dim3 gA((unsigned)std::min<int64_t>((m + 255) / 256, 64), 2 * b);
            launch_k(k_perm_gather<T>, gA, 256, 0, st, A, ld, (int)m, B.Y, nbp, nbp, jpvt, jj, B.plan_src,
                                                 B.plan_n, B.tmp, B.tmpY, B.tmpI);
            launch_k(k_perm_scatter<T>, gA, 256, 0, st, A, ld, (int)m, B.Y, nbp, nbp, jpvt, jj, B.plan_dst,
                                                  B.plan_n, B.tmp, B.tmpY, B.tmpI);
            SKL_LAUNCHED();
            SKL_LAUNCHED();
            tm.end(1, t0);
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
            if (side_pending) {
                SKL_CUDA(cudaStreamWaitEvent(st, evG, 0));
                side_pending = false;
            }
            cudaEvent_t t0 = tm.begin();
            const int* cf = nullptr;
            if (use_chol && !last) {
                chol_panel<T>(A + j + j * ld, ld, M, b, jj, A, B.cg, B.cr1, B.cx1, B.cw, B.tmp, B.V, m,
                              B.Tm, nb, tau, B.part, B.part_cap, B.chol_fail, st);
                cf = B.chol_fail;
            }
            void* args[] = {&A, &ld, &jj, (void*)&M, (void*)&b, &R, &tau_p, &Tm, &ldt, &V,
                            &ldv, &jpvt, &Yp, &ldy, &nbpp, &pp, (void*)&cf};
            launch_cluster<T>((const void*)k_panel<T>, dim3(kQrThreads), psm, st, args);
            tm.end(2, t0);
            trace_phase(st, "qr: panel");
        }
        T* Gj = B.G + j * nbp;
        if (pivoting && !last) {
            // side: GU = G(:, j:m) V ; GUT = GU T ; B = G1 - GUT V1^T
            SKL_CUDA(cudaEventRecord(evV, st));
            SKL_CUDA(cudaStreamWaitEvent(side, evV, 0));
            cudaEvent_t t0 = tms.begin();
            gemm<T>(false, false, nbp, b, M, T(1), Gj, nbp, B.V, m, T(0), B.GU, nbp, B.part2,
                    B.part2_cap, side);
            gemm<T>(false, false, nbp, b, b, T(1), B.GU, nbp, B.Tm, nb, T(0), B.GUT, nbp, nullptr,
                    0, side);
            launch_k(k_copy_block<T>, 16, 256, 0, side, Gj, nbp, B.Bm, nbp, nbp, b);
            SKL_LAUNCHED();
            gemm<T>(false, true, nbp, b, b, T(-1), B.GUT, nbp, B.V, m, T(1), B.Bm, nbp, nullptr, 0,
                    side);
            // G(:, j:m) -= GUT V^T needs only GUT and V: done here, it overlaps W and
            // R12 on the main stream instead of following the next sample QRP (the
            // next panel, which rewrites V, waits for it through evG)
            gemm<T>(false, true, nbp, M, b, T(-1), B.GUT, nbp, B.V, m, T(1), Gj, nbp, nullptr, 0,
                    side);
            SKL_CUDA(cudaEventRecord(evG, side));
            tms.end(7, t0);
        }
        const int N2 = N - b;
        T* Atr = A + j + (j + b) * ld;
        if (N2 > 0) {
            // W = V^T A_trail ; Z = T^T W
            cudaEvent_t t0 = tm.begin();
            if constexpr (std::is_same<T, float>::value) {
                // tensor cores (tcgen05, 3xTF32): W is on the panel chain's critical path
                vta_product(tc_qr_enabled(), M, N2, b, B.V, m, Atr, ld, B.W, B.tcs, B.tcs_floats,
                            status, st);
            } else {
                gemm<T>(true, false, b, N2, M, T(1), B.V, m, Atr, ld, T(0), B.W, b, B.part,
                        B.part_cap, st);
            }
            tm.end(4, t0);
            t0 = tm.begin();
            gemm<T>(true, false, b, N2, b, T(1), B.Tm, nb, B.W, b, T(0), B.Z, b, nullptr, 0, st);
            tm.end(5, t0);
        }
        // with pivoting the first b rows of the trailing update (R12 = A12 - V1 Z)
        // go first and alone: the side stream reads R12 in place while the
        // main stream updates rows b.. of the trailing matrix
        const bool split_update = pivoting && !last;
        if (split_update) {
            if (N2 > 0)
                gemm<T>(false, false, b, N2, b, T(-1), B.V, m, B.Z, b, T(1), Atr, ld, nullptr, 0, st);
            SKL_CUDA(cudaEventRecord(evR, st));
            SKL_CUDA(cudaStreamWaitEvent(side, evR, 0));
            // side: Y2 -= B R12 and the next sample QRP (evY)
            cudaEvent_t t0 = tms.begin();
            if (N2 > 0)
                gemm<T>(false, false, nbp, N2, b, T(-1), B.Bm, nbp, Atr, ld, T(1),
                        B.Y + (j + b) * nbp, nbp, nullptr, 0, side);
            tms.end(7, t0);
            const int64_t jn = j + nb;
            const bool next_last = (jn + nb >= m) || (jn + nb >= d);
            if (jn < mn && !next_last) {
                const int bn = (int)std::min<int64_t>(nb, std::min<int64_t>(d - jn, m - jn));
                // evD: the sample is downdated and the sample QRP is next on the
                // (high-priority) side stream.  The trailing update waits for it:
                // launched first, the update's CTAs would fill every GPC and the
                // QRP's 16-CTA cluster could start only after the update drained;
                // launched after it, the QRP holds one GPC and the two overlap.
                SKL_CUDA(cudaEventRecord(evD, side));
                launch_yqrp(jn, bn, (int)(d - jn), side, tms);
                SKL_CUDA(cudaStreamWaitEvent(st, evD, 0));
            }
            SKL_CUDA(cudaEventRecord(evY, side));
            side_pending = true;
        }
        if (N2 > 0) {
            // A_trail -= V Z (rows b.. when the first b went ahead)
            cudaEvent_t t0 = tm.begin();
            const int r0 = split_update ? b : 0;
            if constexpr (std::is_same<T, float>::value) {
                if (tc_qr_enabled())
                    tc_update(M, N2, b, r0, B.V, m, B.Z, b, Atr, ld, B.tcu, status, st);
                else
                    gemm<T>(false, false, M - r0, N2, b, T(-1), B.V + r0, m, B.Z, b, T(1), Atr + r0, ld,
                            nullptr, 0, st);
            } else {
                gemm<T>(false, false, M - r0, N2, b, T(-1), B.V + r0, m, B.Z, b, T(1), Atr + r0, ld,
                        nullptr, 0, st);
            }
            tm.end(6, t0);
        }
        if (c) {
            cudaEvent_t t0 = tm.begin();
            launch_k(k_qt_w<T>, b, 256, 0, st, B.V, m, M, b, c + j, B.qw);
            launch_k(k_qt_update<T>, (unsigned)std::max<int64_t>(1, (M + 127) / 128), 128, 0, st, 
                B.V, m, M, b, B.Tm, nb, B.qw, c + j);
            SKL_LAUNCHED();
            SKL_LAUNCHED();
            tm.end(3, t0);
        }
    }
    if (side_pending) {
        SKL_CUDA(cudaStreamWaitEvent(st, evG, 0));
        SKL_CUDA(cudaStreamWaitEvent(st, evY, 0));
    }
    tms.finish();
    tm.finish();
}

template <typename T>
void cpqr(T* A, int64_t m, int64_t d, int64_t ld, int* jpvt, T* tau, void* work, unsigned* status,
          cudaStream_t st, double* c, int pivoting, double* qr_prof, int nb_cap)
{
    qr_core<T>(A, m, d, ld, jpvt, tau, work, status, st, c, pivoting != 0, qr_prof, nb_cap);
}

int cpqr_panel_width(int64_t m, int64_t d, int nb_cap)
{
    return qr_plan<float>(m, d, nb_cap).nb;
}

template void cpqr<float>(float*, int64_t, int64_t, int64_t, int*, float*, void*, unsigned*,
                          cudaStream_t, double*, int, double*, int);
template void cpqr<double>(double*, int64_t, int64_t, int64_t, int*, double*, void*, unsigned*,
                           cudaStream_t, double*, int, double*, int);
template size_t cpqr_workspace_bytes<float>(int64_t, int64_t);
template size_t cpqr_workspace_bytes<double>(int64_t, int64_t);

}  // namespace skl
