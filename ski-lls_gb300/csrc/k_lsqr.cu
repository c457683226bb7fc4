// k_lsqr.cu -- preconditioned LSQR on the GPU.
//
// Restates the Paige-Saunders recurrences of lsqr() (src/IterSolver.cpp:160-284)
// for the operator Abar = A * P1 * D * M of LinOP_sparse_preconditioner /
// LinOP_dense_preconditioner (src/IterSolver.cpp:21-108), where P1 selects the
// first `rank` pivoted columns, D is the column equilibration and M = R11^{-1}.
//
// One iteration is five kernels, all reading their scalars from a device
// state block so that the loop runs without host round trips and can be
// captured in a CUDA graph:
//   tri_n   z = D P1 (M v)                 (triangular mat-vec, row-major M)
//   spmv_n  uh = A z - (alpha/beta) uh     (CSR rows / dense columns), beta'
//   spmv_t  t = D P1^T A^T uh / beta'      (CSC columns / dense columns)
//   tri_t   vh = M^T t - (beta'/alpha) vh  (triangular mat-vec, column-major M), alpha'
//   update  Givens rotation, x += (phi/rho) w, w = v - (theta/rho) w, stop test
// u and v are kept unnormalised (uh = beta u, vh = alpha v) so normalisation
// folds into the next product.  Norms are reduced from per-block partials in a
// fixed order (by the last block of spmv_n; tri_t's partials by every block of
// the update kernel, which needs alpha' anyway), so every run is bitwise
// reproducible.
//
// Mixed precision: the products accumulate in float-float (see common.cuh):
// matrix values are stored as (hi, lo) float pairs (8 bytes, like FP64, with
// 48 of FP64's 53 significand bits), the input vectors as (hi, lo) pairs, and
// the scalar recurrences stay in FP64.  On the sparse path the pairs hold the
// equilibrated values A(:, c) / ||A(:, c)||, so no value leaves the float
// range.  The all-FP64 path uses plain double values and DFMA.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "skl_internal.hpp"
#include "launch.cuh"
#include "common.cuh"

namespace skl {

// Scalars every thread of a product kernel needs (ratios, reciprocals, the
// Givens update's coefficients) are formed once by the thread that finalises
// the norm they depend on, not per thread: GB300 issues FP64 at 1/64 of the
// FP32 rate, and a division repeated by every warp of a grid cost several us
// per kernel.
struct LsqrState {
    double alpha, beta, alpha_new, rhobar, phibar, nrm_a, nrm_ar, tol;
    long long it, max_it;
    int done, flag;
    unsigned cnt[4];
    double coef_n;      // alpha / beta: spmv_n's uh = A z - coef_n uh
    double ib;          // 1 / beta:     spmv_t's t = A^T uh / beta
    double coef_t;      // beta / alpha: tri_t's vh = M^T t - coef_t vh
    double up_t1, up_t2, up_ia;   // update: y += t1 w, w = v + t2 w, v = vh / alpha
    float2 coef_n_ff;   // coef_n as a (hi, lo) float pair
};

// beta is final: the ratios spmv_t and tri_t use (one thread)
SKL_DEV void state_after_beta(LsqrState* S, double beta)
{
    S->beta = beta;
    S->ib = beta > 0.0 ? 1.0 / beta : 0.0;
    S->coef_t = S->alpha > 0.0 ? beta / S->alpha : 0.0;
}

// alpha (S->alpha) and beta final for the next spmv_n (one thread)
SKL_DEV void state_coef_n(LsqrState* S)
{
    const double c = S->beta > 0.0 ? S->alpha / S->beta : 0.0;
    S->coef_n = c;
    ff f = ff_from_double(c);
    S->coef_n_ff = make_float2(f.hi, f.lo);
}

// alpha' is final: the Givens rotation and the update's coefficients (one thread)
SKL_DEV void state_update_coefs(LsqrState* S)
{
    const double alpha_old = S->alpha;
    const double beta = S->beta;
    // the reference skips the A^T u step when beta == 0 (IterSolver.cpp:242)
    const double alpha = beta > 0.0 ? S->alpha_new : alpha_old;
    const double rho = sqrt(S->rhobar * S->rhobar + beta * beta);
    const double cs = S->rhobar / rho, sn = beta / rho;
    const double theta = sn * alpha;
    const double phi = cs * S->phibar;
    S->up_t1 = phi / rho;
    S->up_t2 = -theta / rho;
    S->up_ia = alpha > 0.0 ? 1.0 / alpha : 0.0;
}

constexpr int kLThreads = 256;
// Threads per row pair of the triangular products.  r = 4,950 gives 2,475
// pairs of equal length: 17 blocks per SM must be co-resident (16.3 on
// average) for one wave, which 96-thread blocks at <= 40 registers allow;
// 128-thread blocks left a second wave on part of the GPU.
constexpr int kTriThreads = 96;
constexpr int kTriMinBlocks = 17;

// Fixed-order reduction of partials[0..np) by one block; result to *out.
// Eight loads per thread are issued before their (ordered) adds: with 2,475
// partials and 96 threads a load-add-load chain was ~9 us of L2 latency in
// the grid's last block.
SKL_DEV double block_reduce_partials(const double* partials, int np)
{
    __shared__ double red[kLThreads / 32];
    double s = 0.0;
    const int nt = blockDim.x;
    int i = threadIdx.x;
    for (; i + 7 * nt < np; i += 8 * nt) {
        double v[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] = partials[i + k * nt];
#pragma unroll
        for (int k = 0; k < 8; ++k) s += v[k];
    }
    for (; i < np; i += nt) s += partials[i];
    return block_sum(s, red);
}

// Returns true in the last block to arrive (all blocks' partials visible).
SKL_DEV bool arrive_last(unsigned* counter)
{
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned t = atomicAdd(counter, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    return last;
}

template <bool MIXED>
struct VecT {
    using type = double;
};
template <>
struct VecT<true> {
    using type = float2;
};

template <bool MIXED>
SKL_DEV typename VecT<MIXED>::type store_val(double x)
{
    if constexpr (MIXED) {
        ff f = ff_from_double(x);
        return make_float2(f.hi, f.lo);
    } else {
        return x;
    }
}

template <bool MIXED>
struct Acc {
    ff a{0.f, 0.f};
    SKL_DEV void fma_mv(float2 m, float2 x) { ff_fma(a, ff{m.x, m.y}, ff{x.x, x.y}); }
    SKL_DEV void fma_f(float m, float2 x) { ff_fma_f(a, m, ff{x.x, x.y}); }
    SKL_DEV void add(const Acc& o) { ff_add(a, o.a); }
    SKL_DEV Acc shfl_xor(int o) const { Acc r; r.a = ff_shfl_xor(a, o); return r; }
    SKL_DEV double value() const { return ff_to_double(a); }
};
template <>
struct Acc<false> {
    double a = 0.0;
    SKL_DEV void fma_mv(double m, double x) { a = fma(m, x, a); }
    SKL_DEV void fma_f(double m, double x) { a = fma(m, x, a); }
    SKL_DEV void add(const Acc& o) { a += o.a; }
    SKL_DEV Acc shfl_xor(int o) const { Acc r; r.a = __shfl_xor_sync(0xffffffffu, a, o); return r; }
    SKL_DEV double value() const { return a; }
};

template <bool MIXED>
using MatT = typename std::conditional<MIXED, float, double>::type;
template <bool MIXED>
using ValT = typename VecT<MIXED>::type;   // stored A values: float2 (hi,lo) or double

// ------------------------------------------------------- triangular dots --
// Partial dot of M[j0:j1] (contiguous) with v[j0:j1] for one thread of a block
// that strides 4-element chunks by `nthr`: 16-byte loads, two independent
// accumulators.  Head/tail elements (before the first 4-element boundary and
// after the last whole chunk) are taken by the first threads.  The row start
// must be 4-element aligned in memory (ldm is a multiple of 4).
template <bool MIXED>
SKL_DEV Acc<MIXED> thread_dot_seg(const MatT<MIXED>* __restrict__ M, const ValT<MIXED>* __restrict__ v,
                                  int j0, int j1, int t, int nthr)
{
    Acc<MIXED> a0, a1;
    const int jb = min(j1, (j0 + 3) & ~3);
    if (t < jb - j0) a0.fma_f(M[j0 + t], v[j0 + t]);
    const int nch = (j1 - jb) >> 2;
    const int je = jb + (nch << 2);
    // Chunks c, c + nthr, ... in order; two chunks per pass so that two
    // 16-byte matrix loads per thread are in flight.
    if constexpr (MIXED) {
        const float4* M4 = reinterpret_cast<const float4*>(M + jb);
        const float4* v4 = reinterpret_cast<const float4*>(v + jb);   // 2 elements per float4
        auto chunk = [&](const float4& m0, const float4& x0, const float4& x1) {
            a0.fma_f(m0.x, make_float2(x0.x, x0.y));
            a1.fma_f(m0.y, make_float2(x0.z, x0.w));
            a0.fma_f(m0.z, make_float2(x1.x, x1.y));
            a1.fma_f(m0.w, make_float2(x1.z, x1.w));
        };
        int c = t;
        for (; c + nthr < nch; c += 2 * nthr) {
            const int c2 = c + nthr;
            const float4 m0 = M4[c], m1 = M4[c2];
            const float4 x0 = v4[2 * c], x1 = v4[2 * c + 1];
            const float4 y0 = v4[2 * c2], y1 = v4[2 * c2 + 1];
            chunk(m0, x0, x1);
            chunk(m1, y0, y1);
        }
        if (c < nch) chunk(M4[c], v4[2 * c], v4[2 * c + 1]);
    } else {
        const double2* M2 = reinterpret_cast<const double2*>(M + jb);
        const double2* v2 = reinterpret_cast<const double2*>(v + jb);
        auto chunk = [&](int c) {
            const double2 m0 = M2[2 * c], m1 = M2[2 * c + 1];
            const double2 x0 = v2[2 * c], x1 = v2[2 * c + 1];
            a0.fma_f(m0.x, x0.x);
            a1.fma_f(m0.y, x0.y);
            a0.fma_f(m1.x, x1.x);
            a1.fma_f(m1.y, x1.y);
        };
        for (int c = t; c < nch; c += nthr) chunk(c);
    }
    if (t < j1 - je) a1.fma_f(M[je + t], v[je + t]);
    a0.add(a1);
    return a0;
}

// Fixed-order block reduction of two accumulators (all threads call it).
template <bool MIXED>
SKL_DEV void block_reduce2(Acc<MIXED>& a, Acc<MIXED>& b, Acc<MIXED>* sm)
{
    constexpr int NW = kTriThreads / 32;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a.add(a.shfl_xor(o));
        b.add(b.shfl_xor(o));
    }
    if (lane == 0) {
        sm[wid] = a;
        sm[NW + wid] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < NW; ++q) {
            sm[0].add(sm[q]);
            sm[NW].add(sm[NW + q]);
        }
    }
    __syncthreads();
    a = sm[0];
    b = sm[NW];
}

// ------------------------------------------------------------- tri_n -----
// z[cols[i]] = colscale[cols[i]] * sum_{j>=i} M[i][j] v[j]   (Mr row-major;
// colscale == nullptr: no scale, the stored values are already equilibrated)
// One block per row pair (i, r-1-i): every block reads ~r+1 entries.
template <bool MIXED>
__global__ void __launch_bounds__(kTriThreads, MIXED ? kTriMinBlocks : 1)
k_tri_n(const MatT<MIXED>* __restrict__ Mr, int64_t ldm, int r, const ValT<MIXED>* __restrict__ v,
        const int* __restrict__ cols, const double* __restrict__ colscale,
        ValT<MIXED>* __restrict__ z, const LsqrState* __restrict__ S, int plain_out,
        double* __restrict__ zplain)
{
    pdl_wait();
    if (S && S->done) return;
    __shared__ Acc<MIXED> sm[2 * kTriThreads / 32];
    const int npairs = (r + 1) / 2;
    for (int pidx = blockIdx.x; pidx < npairs; pidx += gridDim.x) {
        const int i1 = pidx, i2 = r - 1 - pidx;
        Acc<MIXED> a = thread_dot_seg<MIXED>(Mr + (int64_t)i1 * ldm, v, i1, r, threadIdx.x, kTriThreads);
        Acc<MIXED> b;
        if (i2 != i1) b = thread_dot_seg<MIXED>(Mr + (int64_t)i2 * ldm, v, i2, r, threadIdx.x, kTriThreads);
        block_reduce2<MIXED>(a, b, sm);
        if (threadIdx.x == 0) {
            int c = cols[i1];
            double val = (colscale ? colscale[c] : 1.0) * a.value();
            if (plain_out) zplain[c] = val;
            else z[c] = store_val<MIXED>(val);
            if (i2 != i1) {
                c = cols[i2];
                val = (colscale ? colscale[c] : 1.0) * b.value();
                if (plain_out) zplain[c] = val;
                else z[c] = store_val<MIXED>(val);
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------- tri_t -----
// vh[j] = sum_{i<=j} M[i][j] t[i] - coef * vh[j], coef = beta'/alpha (0 at init)
template <bool MIXED>
__global__ void __launch_bounds__(kTriThreads, MIXED ? kTriMinBlocks : 1)
k_tri_t(const MatT<MIXED>* __restrict__ Mc, int64_t ldm, int r, const ValT<MIXED>* __restrict__ t,
        double* __restrict__ vh, LsqrState* __restrict__ S, int init, double* __restrict__ partials)
{
    pdl_wait();
    if (S->done) return;
    __shared__ Acc<MIXED> sm[2 * kTriThreads / 32];
    const double coef = init ? 0.0 : S->coef_t;
    const int npairs = (r + 1) / 2;
    double ss = 0.0;
    for (int pidx = blockIdx.x; pidx < npairs; pidx += gridDim.x) {
        const int j1 = pidx, j2 = r - 1 - pidx;
        // the old vh of both columns, loaded before the dots so the epilogue
        // does not wait on memory
        double o1 = 0.0, o2 = 0.0;
        if (threadIdx.x == 0) {
            o1 = vh[j1];
            if (j2 != j1) o2 = vh[j2];
        }
        Acc<MIXED> a = thread_dot_seg<MIXED>(Mc + (int64_t)j1 * ldm, t, 0, j1 + 1, threadIdx.x, kTriThreads);
        Acc<MIXED> b;
        if (j2 != j1) b = thread_dot_seg<MIXED>(Mc + (int64_t)j2 * ldm, t, 0, j2 + 1, threadIdx.x, kTriThreads);
        block_reduce2<MIXED>(a, b, sm);
        if (threadIdx.x == 0) {
            double nv = a.value() - coef * o1;
            vh[j1] = nv;
            ss += nv * nv;
            if (j2 != j1) {
                nv = b.value() - coef * o2;
                vh[j2] = nv;
                ss += nv * nv;
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) partials[blockIdx.x] = ss;
    // in the iterations k_lsqr_update reduces the partials itself (every block,
    // fixed order); only the initial product finalises alpha here
    if (init && arrive_last(&S->cnt[1])) {
        double tot = block_reduce_partials(partials, gridDim.x);
        if (threadIdx.x == 0) {
            S->alpha_new = sqrt(tot);
            S->cnt[1] = 0;
        }
    }
}

// Loads of U (index, value) entries p, p+L, ..., p+(U-1)L of one row or
// column, predicated on q < p1 (index 0 and value 0 past the end, so the
// matching gather reads a valid element and contributes nothing).
template <bool MIXED, int L, int U>
SKL_DEV void load_group(const int* __restrict__ idx, const ValT<MIXED>* __restrict__ val, int p,
                        int p1, int (&ii)[U], ValT<MIXED> (&aa)[U])
{
#pragma unroll
    for (int k = 0; k < U; ++k) {
        const int q = p + k * L;
        const bool ok = q < p1;
        ii[k] = ok ? idx[q] : 0;
        aa[k] = ok ? val[q] : ValT<MIXED>{};
    }
}

template <bool MIXED, int L>
SKL_DEV void load_group4(const int* __restrict__ idx, const ValT<MIXED>* __restrict__ val, int p,
                         int p1, int (&ii)[4], ValT<MIXED> (&aa)[4])
{
    load_group<MIXED, L, 4>(idx, val, p, p1, ii, aa);
}

// The old u of one row for spmv_n's recurrence: a float pair read from us
// on the mixed path (uh is not kept there), the FP64 uh otherwise.
template <bool MIXED>
struct UOld {
    ff v{0.f, 0.f};
    SKL_DEV static UOld load(const double*, const float2* us, int i)
    {
        UOld o;
        const float2 t = us[i];
        o.v = ff{t.x, t.y};
        return o;
    }
};
template <>
struct UOld<false> {
    double v = 0.0;
    SKL_DEV static UOld load(const double* uh, const double*, int i)
    {
        UOld o;
        o.v = uh[i];
        return o;
    }
};

// ---------------------------------------------------------- spmv_n (CSR) --
// uh[i] = sum_j A[i][j] z[j] - coef * uh[i], coef = alpha/beta (0 at init with
// z = 0 replaced by rhs b);  usplit = split(uh);  beta' = ||uh||.
constexpr int kRowTile = 512;   // rows whose pointers a block stages at a time

template <bool MIXED, int L>
__global__ void __launch_bounds__(kLThreads)
k_spmv_n_csr(const int* __restrict__ rp, const int* __restrict__ ci, const ValT<MIXED>* __restrict__ cv,
             int n, int rows_per_block, const ValT<MIXED>* __restrict__ zg, int d_stage,
             double* __restrict__ uh, ValT<MIXED>* __restrict__ us, LsqrState* __restrict__ S,
             double* __restrict__ partials)
{
    pdl_wait();
    using V = ValT<MIXED>;
    if (S->done) return;
    __shared__ double wsum[kLThreads / 32];
    __shared__ int rps[kRowTile + 1];
    // z is gathered at random columns: stage it in shared memory when it fits
    extern __shared__ __align__(16) unsigned char zsm_raw[];
    const V* z = zg;
    if (d_stage > 0) {
        V* zs = reinterpret_cast<V*>(zsm_raw);
        for (int j = threadIdx.x; j < d_stage; j += blockDim.x) zs[j] = zg[j];
        z = zs;
    }
    // Each warp owns 32/L consecutive row slots per pass; the pass count is
    // uniform across the warp so the full-mask shuffles below always see all
    // 32 lanes (groups past the last row contribute zero).  Rows are software
    // pipelined: the first four (index, value) loads per lane and the old
    // uh of the next pass's row are issued before the current row's gathers
    // and arithmetic, and the row pointers come from shared memory, so a pass
    // waits on one memory round trip instead of three.
    const int lane = threadIdx.x % L;
    const int grp = threadIdx.x / L;
    const int ngrp = kLThreads / L;
    const double coef = S->coef_n;
    const ff coef_ff{S->coef_n_ff.x, S->coef_n_ff.y};
    const int r0 = blockIdx.x * rows_per_block;
    const int r1 = min(n, r0 + rows_per_block);
    const int warp_grp0 = (threadIdx.x >> 5) * (32 / L);
    double ss = 0.0;
    ff ssf{0.f, 0.f};
    for (int t0 = r0; t0 < r1; t0 += kRowTile) {
        const int t1 = min(r1, t0 + kRowTile);
        __syncthreads();   // z staged; the previous tile's pointers are no longer read
        for (int q = threadIdx.x; q <= t1 - t0; q += blockDim.x) rps[q] = rp[t0 + q];
        __syncthreads();
        int i = t0 + grp;
        bool act = i < t1;
        int pb = 0, p1 = 0;
        int cc[4];
        V aa[4];
        UOld<MIXED> uo;
        if (act) {
            pb = rps[i - t0] + lane;
            p1 = rps[i - t0 + 1];
            if (lane == 0) uo = UOld<MIXED>::load(uh, us, i);
        }
        load_group4<MIXED, L>(ci, cv, pb, p1, cc, aa);
        for (int base = t0 + warp_grp0; base < t1; base += ngrp) {
            const int ni = i + ngrp;
            const bool nact = ni < t1;
            int npb = 0, np1 = 0;
            int nc[4];
            V na[4];
            UOld<MIXED> nuo;
            if (nact) {
                npb = rps[ni - t0] + lane;
                np1 = rps[ni - t0 + 1];
                if (lane == 0) nuo = UOld<MIXED>::load(uh, us, ni);
            }
            load_group4<MIXED, L>(ci, cv, npb, np1, nc, na);
            Acc<MIXED> acc, acc2;
            {
                V zz[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) zz[k] = z[cc[k]];
                acc.fma_mv(aa[0], zz[0]);
                acc2.fma_mv(aa[1], zz[1]);
                acc.fma_mv(aa[2], zz[2]);
                acc2.fma_mv(aa[3], zz[3]);
            }
            // rows longer than 4L: the remaining groups of four, unpipelined
            for (int p = pb + 4 * L; p < p1; p += 4 * L) {
                int c2[4];
                V a2[4];
                load_group4<MIXED, L>(ci, cv, p, p1, c2, a2);
                V zz[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) zz[k] = z[c2[k]];
                acc.fma_mv(a2[0], zz[0]);
                acc2.fma_mv(a2[1], zz[1]);
                acc.fma_mv(a2[2], zz[2]);
                acc2.fma_mv(a2[3], zz[3]);
            }
            acc.add(acc2);
#pragma unroll
            for (int o = L / 2; o > 0; o >>= 1) acc.add(acc.shfl_xor(o));
            if (act && lane == 0) {
                if constexpr (MIXED) {
                    // float-float throughout: uh lives only as the pair us
                    ff nv = acc.a;
                    ff_fma(nv, ff{-coef_ff.hi, -coef_ff.lo}, uo.v);
                    us[i] = make_float2(nv.hi, nv.lo);
                    ff_fma(ssf, nv, nv);
                } else {
                    double nv = acc.value() - coef * uo.v;
                    uh[i] = nv;
                    us[i] = store_val<MIXED>(nv);
                    ss += nv * nv;
                }
            }
            i = ni;
            act = nact;
            pb = npb;
            p1 = np1;
            uo = nuo;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                cc[k] = nc[k];
                aa[k] = na[k];
            }
        }
    }
    if constexpr (MIXED) ss = ff_to_double(ssf);
    ss = warp_sum(ss);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = ss;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int q = 0; q < kLThreads / 32; ++q) s += wsum[q];
        partials[blockIdx.x] = s;
    }
    if (arrive_last(&S->cnt[0])) {
        double tot = block_reduce_partials(partials, gridDim.x);
        if (threadIdx.x == 0) {
            state_after_beta(S, sqrt(tot));
            S->cnt[0] = 0;
        }
    }
}

// --------------------------------------------------------- spmv_t (CSC) --
// t[i] = colscale[c] * (sum_{p in col c} A[p] u[row p]) / beta,  c = cols[i]
// (colscale == nullptr: no scale)
// L lanes per column, kTU entries per lane per step; the (index, value) loads
// of the next step are issued before the gathers of the current step are
// consumed, so the HBM stream of A overlaps the L2 gathers of u.  Each warp
// walks one long column, so the kernel is bound by how many bytes each warp
// keeps in flight: 8 entries per lane per step (12 B each) halves the
// dependent steps per column against 4.
constexpr int kTU = 8;

template <bool MIXED, int L>
__global__ void __launch_bounds__(kLThreads)
k_spmv_t_csc(const int* __restrict__ cp, const int* __restrict__ ri, const ValT<MIXED>* __restrict__ cv,
             const int* __restrict__ cols, const double* __restrict__ colscale, int r,
             const ValT<MIXED>* __restrict__ us, ValT<MIXED>* __restrict__ t,
             const LsqrState* __restrict__ S)
{
    pdl_wait();
    using V = ValT<MIXED>;
    if (S->done) return;
    const int lane = threadIdx.x % L;
    const int g = (blockIdx.x * blockDim.x + threadIdx.x) / L;
    const int ng = (gridDim.x * blockDim.x) / L;
    const int gw0 = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * (32 / L);  // first group of this warp
    const double ib = S->ib;
    // warp-uniform trip count (see k_spmv_n_csr)
    for (int base = gw0; base < r; base += ng) {
        const int i = base + (g - gw0);
        const bool active = i < r;
        Acc<MIXED> acc, acc2;
        int c = 0;
        if (active) {
            c = cols[i];
            const int p1 = cp[c + 1];
            int pb = cp[c] + lane;
            int rr[kTU];
            V aa[kTU];
            load_group<MIXED, L, kTU>(ri, cv, pb, p1, rr, aa);
            while (pb < p1) {
                V uu[kTU];
#pragma unroll
                for (int k = 0; k < kTU; ++k) uu[k] = us[rr[k]];
                const int pn = pb + kTU * L;
                int rn[kTU];
                V an[kTU];
                load_group<MIXED, L, kTU>(ri, cv, pn, p1, rn, an);
#pragma unroll
                for (int k = 0; k < kTU; k += 2) {
                    acc.fma_mv(aa[k], uu[k]);
                    acc2.fma_mv(aa[k + 1], uu[k + 1]);
                }
#pragma unroll
                for (int k = 0; k < kTU; ++k) {
                    rr[k] = rn[k];
                    aa[k] = an[k];
                }
                pb = pn;
            }
        }
        acc.add(acc2);
#pragma unroll
        for (int o = L / 2; o > 0; o >>= 1) acc.add(acc.shfl_xor(o));
        if (active && lane == 0)
            t[i] = store_val<MIXED>((colscale ? colscale[c] : 1.0) * acc.value() * ib);
    }
}

// ------------------------------------------------- dense A (column-major) --
// spmv_n: uh = A(:, cols) z(cols) - coef uh.  A block covers 512 rows (two
// per thread, 256 apart, so each column's loads stay warp-contiguous) and the
// columns of one chunk (at most kDenseChunk), whose indices and z entries it
// first stages in shared memory; four columns per step keep eight independent
// loads in flight per thread.  Chunk partials are combined by
// spmv_n_dense_reduce.
constexpr int kDnRows = 2 * kLThreads;
constexpr int kDenseChunk = 512;

template <bool MIXED>
__global__ void __launch_bounds__(kLThreads)
k_spmv_n_dense(const ValT<MIXED>* __restrict__ A, int64_t lda, int n, const int* __restrict__ cols,
               int r, int chunk, const ValT<MIXED>* __restrict__ z, double* __restrict__ part,
               const LsqrState* __restrict__ S)
{
    pdl_wait();
    using V = ValT<MIXED>;
    if (S->done) return;
    __shared__ int scol[kDenseChunk];
    __shared__ V sz[kDenseChunk];
    const int c0 = blockIdx.y * chunk, nc = min(r - c0, chunk);
    for (int k = threadIdx.x; k < nc; k += kLThreads) {
        const int col = cols[c0 + k];
        scol[k] = col;
        sz[k] = z[col];
    }
    __syncthreads();
    const int i0 = blockIdx.x * kDnRows + threadIdx.x, i1 = i0 + kLThreads;
    if (i0 >= n) return;
    const int j1 = i1 < n ? i1 : i0;   // a row past the end re-reads row i0; its sum is not stored
    Acc<MIXED> a0, a1;
    int k = 0;
    for (; k + 4 <= nc; k += 4) {
        V x0[4], x1[4], zz[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const V* col = A + (int64_t)scol[k + u] * lda;
            x0[u] = col[i0];
            x1[u] = col[j1];
            zz[u] = sz[k + u];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            a0.fma_mv(x0[u], zz[u]);
            a1.fma_mv(x1[u], zz[u]);
        }
    }
    for (; k < nc; ++k) {
        const V* col = A + (int64_t)scol[k] * lda;
        const V zz = sz[k];
        a0.fma_mv(col[i0], zz);
        a1.fma_mv(col[j1], zz);
    }
    double* out = part + (int64_t)blockIdx.y * n;
    out[i0] = a0.value();
    if (i1 < n) out[i1] = a1.value();
}

template <bool MIXED>
__global__ void __launch_bounds__(kLThreads)
k_spmv_n_dense_reduce(const double* __restrict__ part, int nchunks, int n, double* __restrict__ uh,
                      ValT<MIXED>* __restrict__ us, LsqrState* __restrict__ S,
                      double* __restrict__ partials)
{
    pdl_wait();
    if (S->done) return;
    __shared__ double red[kLThreads / 32];
    const double coef = S->coef_n;
    double ss = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int q = 0; q < nchunks; ++q) s += part[(int64_t)q * n + i];
        double nv = s - coef * uh[i];
        uh[i] = nv;
        us[i] = store_val<MIXED>(nv);
        ss += nv * nv;
    }
    ss = block_sum(ss, red);
    if (threadIdx.x == 0) partials[blockIdx.x] = ss;
    if (arrive_last(&S->cnt[0])) {
        double tot = block_reduce_partials(partials, gridDim.x);
        if (threadIdx.x == 0) {
            state_after_beta(S, sqrt(tot));
            S->cnt[0] = 0;
        }
    }
}

// spmv_t: t(i) = colscale(c) A(:, c)^T u / beta for c = cols[i], four
// columns per block: each thread reads u once per row pair for all four
// columns, so u costs a quarter of A's bytes; two rows per step keep ten
// independent loads in flight per thread.
constexpr int kDtCols = 4;

template <bool MIXED>
__global__ void __launch_bounds__(kLThreads)
k_spmv_t_dense(const ValT<MIXED>* __restrict__ A, int64_t lda, int n, const int* __restrict__ cols,
               const double* __restrict__ colscale, int r, const ValT<MIXED>* __restrict__ us,
               ValT<MIXED>* __restrict__ t, const LsqrState* __restrict__ S)
{
    pdl_wait();
    using V = ValT<MIXED>;
    if (S->done) return;
    __shared__ Acc<MIXED> red[kDtCols][kLThreads / 32];
    const double ib = S->ib;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int g = blockIdx.x; g * kDtCols < r; g += gridDim.x) {
        const int i0 = g * kDtCols;
        const int nc = min(kDtCols, r - i0);
        const V* colp[kDtCols];
#pragma unroll
        for (int u = 0; u < kDtCols; ++u) colp[u] = A + (int64_t)cols[i0 + min(u, nc - 1)] * lda;
        Acc<MIXED> acc[kDtCols];
        int q = threadIdx.x;
        for (; q + kLThreads < n; q += 2 * kLThreads) {
            const V u0 = us[q], u1 = us[q + kLThreads];
            V x0[kDtCols], x1[kDtCols];
#pragma unroll
            for (int u = 0; u < kDtCols; ++u) {
                x0[u] = colp[u][q];
                x1[u] = colp[u][q + kLThreads];
            }
#pragma unroll
            for (int u = 0; u < kDtCols; ++u) {
                acc[u].fma_mv(x0[u], u0);
                acc[u].fma_mv(x1[u], u1);
            }
        }
        if (q < n) {
            const V u0 = us[q];
#pragma unroll
            for (int u = 0; u < kDtCols; ++u) acc[u].fma_mv(colp[u][q], u0);
        }
#pragma unroll
        for (int u = 0; u < kDtCols; ++u) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc[u].add(acc[u].shfl_xor(o));
            if (lane == 0) red[u][warp] = acc[u];
        }
        __syncthreads();
        if (threadIdx.x < nc) {
            const int u = threadIdx.x;
            Acc<MIXED> s = red[u][0];
            for (int w = 1; w < kLThreads / 32; ++w) s.add(red[u][w]);
            const int c = cols[i0 + u];
            t[i0 + u] = store_val<MIXED>((colscale ? colscale[c] : 1.0) * s.value() * ib);
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- init --
// uh = b, usplit = split(b), beta = ||b||
template <bool MIXED>
__global__ void __launch_bounds__(kLThreads)
k_lsqr_init_u(const double* __restrict__ b, int n, double* __restrict__ uh,
              ValT<MIXED>* __restrict__ us, LsqrState* __restrict__ S, double* __restrict__ partials)
{
    pdl_wait();
    __shared__ double red[kLThreads / 32];
    double ss = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double x = b[i];
        uh[i] = x;
        us[i] = store_val<MIXED>(x);
        ss += x * x;
    }
    ss = block_sum(ss, red);
    if (threadIdx.x == 0) partials[blockIdx.x] = ss;
    if (arrive_last(&S->cnt[0])) {
        double tot = block_reduce_partials(partials, gridDim.x);
        if (threadIdx.x == 0) {
            state_after_beta(S, sqrt(tot));
            S->cnt[0] = 0;
        }
    }
}

// After the init products: alpha = ||vh||, v = vh/alpha, w = v, y = 0.
template <bool MIXED>
__global__ void __launch_bounds__(kLThreads)
k_lsqr_init_v(int r, double* __restrict__ vh, ValT<MIXED>* __restrict__ vs, double* __restrict__ w,
              double* __restrict__ y, LsqrState* __restrict__ S)
{
    pdl_wait();
    const double alpha = S->alpha_new;
    const double beta = S->beta;
    const double ia = alpha > 0.0 ? 1.0 / alpha : 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < r; i += gridDim.x * blockDim.x) {
        double v = vh[i] * ia;
        vs[i] = store_val<MIXED>(v);
        w[i] = v;
        y[i] = 0.0;
    }
    if (arrive_last(&S->cnt[2])) {
        if (threadIdx.x == 0) {
            S->alpha = alpha;
            S->rhobar = alpha;
            S->phibar = beta;
            S->nrm_a = 0.0;
            S->it = 0;
            S->flag = 1;
            S->done = (alpha * beta == 0.0) ? 1 : 0;
            if (S->done) S->flag = 0;
            state_coef_n(S);
            S->cnt[2] = 0;
        }
    }
}

// ------------------------------------------------------------- update ---
template <bool MIXED>
__global__ void __launch_bounds__(kLThreads)
k_lsqr_update(int r, const double* __restrict__ vh, ValT<MIXED>* __restrict__ vs,
              double* __restrict__ w, double* __restrict__ y, LsqrState* __restrict__ S,
              const double* __restrict__ partials, int npart)
{
    pdl_wait();
    if (S->done) return;
    // alpha' = ||vh|| from tri_t's per-block partials, reduced by every block in
    // the same fixed order (so every block agrees bit for bit), then the
    // Givens coefficients by one thread
    __shared__ double s_coef[3];
    const double alpha_new = sqrt(block_reduce_partials(partials, npart));
    if (threadIdx.x == 0) {
        S->alpha_new = alpha_new;   // same value from every block
        state_update_coefs(S);
        s_coef[0] = S->up_t1;
        s_coef[1] = S->up_t2;
        s_coef[2] = S->up_ia;
    }
    __syncthreads();
    const double beta = S->beta;
    const double t1 = s_coef[0], t2 = s_coef[1], ia = s_coef[2];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < r; i += gridDim.x * blockDim.x) {
        double v = (beta > 0.0) ? vh[i] * ia : 0.0;
        if (beta > 0.0) vs[i] = store_val<MIXED>(v);
        double wi = w[i];
        y[i] += t1 * wi;
        w[i] = t2 * wi + v;
    }
    if (arrive_last(&S->cnt[3])) {
        if (threadIdx.x == 0) {
            const double alpha_old = S->alpha;
            const double alpha = beta > 0.0 ? S->alpha_new : alpha_old;
            const double rho = sqrt(S->rhobar * S->rhobar + beta * beta);
            const double cs = S->rhobar / rho, sn = beta / rho;
            double nrm_a = S->nrm_a;
            if (beta > 0.0) nrm_a = sqrt(nrm_a * nrm_a + alpha_old * alpha_old + beta * beta);
            const double phibar = sn * S->phibar;
            S->rhobar = -cs * alpha;
            S->phibar = phibar;
            S->nrm_a = nrm_a;
            S->alpha = alpha;
            state_coef_n(S);
            S->it += 1;
            const double nrm_ar = phibar * alpha * fabs(cs);
            S->nrm_ar = nrm_ar;
            if (nrm_ar < S->tol * nrm_a * phibar) {
                S->done = 1;
                S->flag = 0;
            } else if (S->it >= S->max_it) {
                S->done = 1;
                S->flag = 1;
            }
            S->cnt[3] = 0;
        }
    }
}

// ------------------------------------------------------------ host side --
struct LsqrBufs {
    LsqrState* S;
    double *uh, *vh, *w, *y, *partials, *dpart;
    void *us, *vs, *t, *z;
    int nparts;
    int dense_chunk;            // columns per block of the dense A z
};

static int sm_count_lsqr()
{
    static const int v = [] {
        int dev = 0, s = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&s, cudaDevAttrMultiProcessorCount, dev);
        return s > 0 ? s : 148;
    }();
    return v;
}

// lanes per row/column so that each lane handles about four nonzeros
static int lanes_for(double avg)
{
    if (avg >= 96) return 32;
    if (avg >= 40) return 16;
    if (avg >= 16) return 8;
    return 4;
}

static const int kRowsPerBlock = 64;

// Columns per block of the dense A z: as many column chunks as keep the grid
// (row blocks x chunks) within one wave of resident blocks, so no second,
// mostly idle wave trails the product; a multiple of 4, at most kDenseChunk.
static int dense_n_chunk(const LsqrProblem& P)
{
    static const int per_sm = [] {
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_spmv_n_dense<true>, kLThreads, 0);
        return b > 0 ? b : 4;
    }();
    const int64_t rb = (P.n + kDnRows - 1) / kDnRows;
    const int64_t slots = (int64_t)sm_count_lsqr() * per_sm;
    const int64_t nch = std::max<int64_t>(1, slots / std::max<int64_t>(rb, 1));
    int64_t c = (P.r + nch - 1) / nch;
    c = (c + 3) & ~(int64_t)3;
    return (int)std::max<int64_t>(4, std::min<int64_t>(c, kDenseChunk));
}

static int64_t spmv_n_blocks(const LsqrProblem& P)
{
    if (P.Ad) return (P.n + kDnRows - 1) / kDnRows;
    return (P.n + kRowsPerBlock - 1) / kRowsPerBlock;   // upper bound on the grid
}

size_t lsqr_workspace_bytes(const LsqrProblem& P)
{
    const size_t vs = P.precision == SKL_PREC_MIXED ? sizeof(float2) : sizeof(double);
    size_t b = sizeof(LsqrState) + 256;
    b += 2 * (P.n * sizeof(double) + 256);                   // uh, us
    b += P.n * vs + 256;
    b += 4 * (P.r * sizeof(double) + 256);                   // vh, w, y, spare
    b += 2 * (P.r * vs + 256);                               // vs, t
    b += P.d * vs + 256;                                     // z
    int64_t nb = spmv_n_blocks(P);
    b += (nb + 4096) * sizeof(double) + 256;                 // partials
    if (P.Ad) {
        const int c = dense_n_chunk(P);
        b += (size_t)((P.r + c - 1) / c) * P.n * sizeof(double) + 256;
    }
    return b;
}

static LsqrBufs carve(const LsqrProblem& P, void* work)
{
    char* base = (char*)work;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        void* r = base + off;
        off += (bytes + 255) & ~(size_t)255;
        return r;
    };
    const size_t vsz = P.precision == SKL_PREC_MIXED ? sizeof(float2) : sizeof(double);
    LsqrBufs B;
    B.S = (LsqrState*)take(sizeof(LsqrState));
    B.uh = (double*)take(P.n * sizeof(double));
    B.us = take(P.n * vsz);
    B.vh = (double*)take(P.r * sizeof(double));
    B.w = (double*)take(P.r * sizeof(double));
    B.y = (double*)take(P.r * sizeof(double));
    B.vs = take(P.r * vsz);
    B.t = take(P.r * vsz);
    B.z = take(P.d * vsz);
    int64_t nb = spmv_n_blocks(P);
    B.nparts = (int)(nb + 4096);
    B.partials = (double*)take(B.nparts * sizeof(double));
    B.dense_chunk = P.Ad ? dense_n_chunk(P) : 0;
    B.dpart = P.Ad ? (double*)take((size_t)((P.r + B.dense_chunk - 1) / B.dense_chunk) * P.n * sizeof(double))
                   : nullptr;
    return B;
}

template <bool MIXED>
static void launch_spmv_n(const LsqrProblem& P, LsqrBufs& B, cudaStream_t st)
{
    using V = ValT<MIXED>;
    if (P.Ad) {
        const int chunk = B.dense_chunk;
        const int nchunks = (int)((P.r + chunk - 1) / chunk);
        dim3 g((unsigned)((P.n + kDnRows - 1) / kDnRows), nchunks);
        launch_k(k_spmv_n_dense<MIXED>, g, kLThreads, 0, st, (const V*)P.Ad, P.lda, (int)P.n, P.cols,
                                                       (int)P.r, chunk, (const V*)B.z, B.dpart, B.S);
        launch_k(k_spmv_n_dense_reduce<MIXED>, (unsigned)std::min<int64_t>((P.n + 255) / 256, 1024), kLThreads, 0, st, B.dpart, nchunks, (int)P.n, B.uh, (V*)B.us, B.S,
                                                B.partials);
        SKL_LAUNCHED();
        SKL_LAUNCHED();
        return;
    }
    const double avg = P.n ? (double)P.nnz / P.n : 0.0;
    const int L = P.lanes_n ? P.lanes_n : lanes_for(avg);
    // z staged in shared memory (<= 96 KB); blocks sized to ~4 per SM
    const size_t zbytes = (size_t)P.d * sizeof(V);
    const int stage = zbytes <= 96 * 1024 ? (int)P.d : 0;
    const size_t smem = stage ? zbytes : 0;
    int rpb = kRowsPerBlock;
    if (stage) rpb = (int)std::max<int64_t>(kRowsPerBlock, (P.n + 152 * 4 - 1) / (152 * 4));
    const unsigned g = (unsigned)((P.n + rpb - 1) / rpb);
#define SPMV_N(LL) do { \
        if (smem > 48 * 1024) allow_max_dynamic_smem((const void*)k_spmv_n_csr<MIXED, LL>); \
        launch_k(k_spmv_n_csr<MIXED, LL>, g, kLThreads, smem, st, P.rp, P.ci, (const V*)P.cx, (int)P.n, rpb, (const V*)B.z, stage, B.uh, (V*)B.us, B.S, B.partials); \
    } while (0)
    if (L == 32) SPMV_N(32);
    else if (L == 16) SPMV_N(16);
    else if (L == 8) SPMV_N(8);
    else SPMV_N(4);
#undef SPMV_N
    SKL_LAUNCHED();
}

template <bool MIXED>
static void launch_spmv_t(const LsqrProblem& P, LsqrBufs& B, cudaStream_t st)
{
    using V = ValT<MIXED>;
    if (P.Ad) {
        unsigned g = (unsigned)std::min<int64_t>((P.r + kDtCols - 1) / kDtCols, 152 * 16);
        launch_k(k_spmv_t_dense<MIXED>, g, kLThreads, 0, st, (const V*)P.Ad, P.lda, (int)P.n, P.cols,
                                                       P.opscale, (int)P.r, (const V*)B.us,
                                                       (V*)B.t, B.S);
        SKL_LAUNCHED();
        return;
    }
    const double avg = P.d ? (double)P.nnz / P.d : 0.0;
    const int L = P.lanes_t ? P.lanes_t : lanes_for(avg);
    const int64_t threads = (int64_t)P.r * L;
    unsigned g = (unsigned)std::min<int64_t>((threads + kLThreads - 1) / kLThreads, 152 * 32);
#define SPMV_T(LL) launch_k(k_spmv_t_csc<MIXED, LL>, g, kLThreads, 0, st, P.cp, P.ri, (const V*)P.rx, P.cols, P.opscale, (int)P.r, (const V*)B.us, (V*)B.t, B.S)
    if (L == 32) SPMV_T(32);
    else if (L == 16) SPMV_T(16);
    else if (L == 8) SPMV_T(8);
    else SPMV_T(4);
#undef SPMV_T
    SKL_LAUNCHED();
}

static unsigned tri_blocks(int64_t r)
{
    int64_t pairs = (r + 1) / 2;
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(pairs, 152 * 32));
}

// ev (optional): 8 events, begin/end around M*v, A*z, A^T*u, M^T*t
template <bool MIXED>
static void launch_iteration(const LsqrProblem& P, LsqrBufs& B, cudaStream_t st,
                             cudaEvent_t* ev = nullptr)
{
    using V = ValT<MIXED>;
    using MT = MatT<MIXED>;
    auto mark = [&](int q) {
        if (ev) SKL_CUDA(cudaEventRecordWithFlags(ev[q], st, cudaEventRecordExternal));
    };
    const unsigned gt = tri_blocks(P.r);
    mark(4);
    launch_k(k_tri_n<MIXED>, gt, kTriThreads, 0, st, (const MT*)P.Mrow, P.ldm, (int)P.r, (const V*)B.vs,
                                              P.cols, P.opscale, (V*)B.z, B.S, 0, nullptr);
    SKL_LAUNCHED();
    mark(5);
    mark(0);
    launch_spmv_n<MIXED>(P, B, st);
    mark(1);
    mark(2);
    launch_spmv_t<MIXED>(P, B, st);
    mark(3);
    mark(6);
    launch_k(k_tri_t<MIXED>, gt, kTriThreads, 0, st, (const MT*)P.M, P.ldm, (int)P.r, (const V*)B.t, B.vh,
                                              B.S, 0, B.partials);
    SKL_LAUNCHED();
    mark(7);
    unsigned gu = (unsigned)std::max<int64_t>(1, std::min<int64_t>((P.r + 255) / 256, 152));
    launch_k(k_lsqr_update<MIXED>, gu, kLThreads, 0, st, (int)P.r, B.vh, (V*)B.vs, B.w, B.y, B.S,
                                                   B.partials, (int)gt);
    SKL_LAUNCHED();
}

template <bool MIXED>
static LsqrResult run_impl(const LsqrProblem& P, const double* b, double tol, int64_t max_it,
                           double* y_out, void* work, void* host_pinned, cudaStream_t st,
                           int profile, cudaStream_t capture_stream)
{
    using V = ValT<MIXED>;
    using MT = MatT<MIXED>;
    LsqrBufs B = carve(P, work);
    LsqrState init{};
    init.tol = tol;
    init.max_it = max_it;
    SKL_CUDA(cudaMemcpyAsync(B.S, &init, sizeof(LsqrState), cudaMemcpyHostToDevice, st));
    SKL_CUDA(cudaMemsetAsync(B.z, 0, P.d * sizeof(V), st));
    // beta_1 u_1 = b ; alpha_1 v_1 = Abar^T u_1
    unsigned gi = (unsigned)std::max<int64_t>(1, std::min<int64_t>((P.n + 255) / 256, 1024));
    launch_k(k_lsqr_init_u<MIXED>, gi, kLThreads, 0, st, b, (int)P.n, B.uh, (V*)B.us, B.S, B.partials);
    SKL_LAUNCHED();
    launch_spmv_t<MIXED>(P, B, st);
    const unsigned gt = tri_blocks(P.r);
    launch_k(k_tri_t<MIXED>, gt, kTriThreads, 0, st, (const MT*)P.M, P.ldm, (int)P.r, (const V*)B.t, B.vh,
                                              B.S, 1, B.partials);
    SKL_LAUNCHED();
    unsigned gu = (unsigned)std::max<int64_t>(1, std::min<int64_t>((P.r + 255) / 256, 152));
    launch_k(k_lsqr_init_v<MIXED>, gu, kLThreads, 0, st, (int)P.r, B.vh, (V*)B.vs, B.w, B.y, B.S);
    SKL_LAUNCHED();

    // Capture a block of iterations once, replay until the device says done.
    const int kIterPerGraph = 4;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    // capture on a non-default stream (capture is not allowed on the legacy
    // default stream); the graph is then launched on the caller's stream
    cudaStream_t cap = capture_stream ? capture_stream : st;
    std::vector<cudaEvent_t> pev;
    if (profile) {
        pev.resize(8 * kIterPerGraph);
        for (auto& e : pev) SKL_CUDA(cudaEventCreate(&e));
    }
    SKL_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
    for (int q = 0; q < kIterPerGraph; ++q)
        launch_iteration<MIXED>(P, B, cap, profile ? &pev[8 * q] : nullptr);
    SKL_CUDA(cudaStreamEndCapture(cap, &graph));
    SKL_CUDA(cudaGraphInstantiate(&exec, graph, 0));
    struct Flags { int done; int flag; long long it; };
    volatile LsqrState* hs = (volatile LsqrState*)host_pinned;
    int64_t launched = 0;
    cudaEvent_t ev;
    SKL_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    bool done = false;
    LsqrResult res;
    long long it_prev = 0;
    trace_phase(st, "lsqr: init");
    const auto t_start = std::chrono::steady_clock::now();
    static const double limit_s = [] {
        const char* e = getenv("SKILLS_LSQR_TIMEOUT_S");
        return e ? atof(e) : 60.0;
    }();
    while (!done) {
        // host-side bound: a replay loop that runs past the limit reports a timeout
        if (std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count() > limit_s) {
            cudaEventDestroy(ev);
            cudaGraphExecDestroy(exec);
            cudaGraphDestroy(graph);
            fail(SKL_ERR_TIMEOUT, "LSQR replay loop exceeded its time limit (SKILLS_LSQR_TIMEOUT_S)");
        }
        SKL_CUDA(cudaGraphLaunch(exec, st));
        launched += kIterPerGraph;
        for (int q = 0; q < 5 * kIterPerGraph; ++q) SKL_LAUNCHED();
        SKL_CUDA(cudaMemcpyAsync((void*)hs, B.S, sizeof(LsqrState), cudaMemcpyDeviceToHost, st));
        SKL_CUDA(cudaEventRecord(ev, st));
        SKL_CUDA(cudaEventSynchronize(ev));
        if (profile) {
            // iterations that ran in this replay (later ones returned at entry)
            long long ran = hs->it - it_prev;
            for (long long q = 0; q < ran && q < kIterPerGraph; ++q)
                for (int kk = 0; kk < 4; ++kk) {
                    float ms = 0.f;
                    SKL_CUDA(cudaEventElapsedTime(&ms, pev[8 * q + 2 * kk], pev[8 * q + 2 * kk + 1]));
                    res.prof_ms[kk] += ms;
                    res.prof_launches[kk] += 1;
                }
        }
        it_prev = hs->it;
        done = hs->done != 0 || launched >= max_it + kIterPerGraph;
    }
    for (auto& e : pev) cudaEventDestroy(e);
    trace_phase(st, "lsqr: done");
    res.flag = hs->flag;
    res.it = hs->it;
    SKL_CUDA(cudaEventDestroy(ev));
    SKL_CUDA(cudaGraphExecDestroy(exec));
    SKL_CUDA(cudaGraphDestroy(graph));
    SKL_CUDA(cudaMemcpyAsync(y_out, B.y, P.r * sizeof(double), cudaMemcpyDeviceToDevice, st));
    return res;
}

LsqrResult lsqr_run(const LsqrProblem& P, const double* b, double tol, int64_t max_it, double* y,
                    void* work, unsigned* status, void* host_pinned, cudaStream_t st, int profile,
                    cudaStream_t capture_stream)
{
    (void)status;
    if (P.precision == SKL_PREC_MIXED)
        return run_impl<true>(P, b, tol, max_it, y, work, host_pinned, st, profile, capture_stream);
    return run_impl<false>(P, b, tol, max_it, y, work, host_pinned, st, profile, capture_stream);
}

// ------------------------------------------------------------- tuning --
// Times the CSR product A z and the CSC product A^T u of this problem's matrix
// for each lanes-per-row (column) choice, median of three launches after one
// warm-up, and keeps the fastest in P.lanes_n / P.lanes_t.
void tune_lsqr_products(LsqrProblem& P, void* work, cudaStream_t st)
{
    if (P.Ad || P.n <= 0 || P.r <= 0) return;
    LsqrBufs B = carve(P, work);
    LsqrState init{};
    init.ib = 1.0;
    init.beta = 1.0;
    const size_t vsz = P.precision == SKL_PREC_MIXED ? sizeof(float2) : sizeof(double);
    SKL_CUDA(cudaMemcpyAsync(B.S, &init, sizeof(LsqrState), cudaMemcpyHostToDevice, st));
    SKL_CUDA(cudaMemsetAsync(B.uh, 0, P.n * sizeof(double), st));
    SKL_CUDA(cudaMemsetAsync(B.us, 0, P.n * vsz, st));
    SKL_CUDA(cudaMemsetAsync(B.z, 0, P.d * vsz, st));
    cudaEvent_t e0, e1;
    SKL_CUDA(cudaEventCreate(&e0));
    SKL_CUDA(cudaEventCreate(&e1));
    auto time_it = [&](auto&& launch) {
        launch();
        float t[3];
        for (float& v : t) {
            SKL_CUDA(cudaEventRecord(e0, st));
            launch();
            SKL_CUDA(cudaEventRecord(e1, st));
            SKL_CUDA(cudaEventSynchronize(e1));
            SKL_CUDA(cudaEventElapsedTime(&v, e0, e1));
        }
        std::sort(t, t + 3);
        return t[1];
    };
    const int cand[4] = {4, 8, 16, 32};
    float best_n = 1e30f, best_t = 1e30f;
    int ln = 0, lt = 0;
    for (int L : cand) {
        P.lanes_n = L;
        const float tn = time_it([&] {
            if (P.precision == SKL_PREC_MIXED) launch_spmv_n<true>(P, B, st);
            else launch_spmv_n<false>(P, B, st);
        });
        if (tn < best_n) { best_n = tn; ln = L; }
        P.lanes_t = L;
        const float tt = time_it([&] {
            if (P.precision == SKL_PREC_MIXED) launch_spmv_t<true>(P, B, st);
            else launch_spmv_t<false>(P, B, st);
        });
        if (tt < best_t) { best_t = tt; lt = L; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    P.lanes_n = ln;
    P.lanes_t = lt;
}

// ------------------------------------------------ one product in isolation --
// y = A x ('n', the CSR kernel of spmv_n) or y = A^T x ('t', the CSC kernel of
// spmv_t) with the storage and arithmetic LSQR uses: on the mixed path the
// stored values are A(:, c) * vscale[c], so the input is divided by vscale
// ('n') or the output ('t').  Used to measure the operator's accuracy.
template <bool MIXED>
__global__ void k_prod_in(const double* __restrict__ x, int64_t len, const double* __restrict__ vscale,
                          ValT<MIXED>* __restrict__ out)
{
    pdl_wait();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len;
         i += (int64_t)gridDim.x * blockDim.x)
        out[i] = store_val<MIXED>(vscale ? x[i] / vscale[i] : x[i]);
}

template <bool MIXED>
__global__ void k_prod_out(const ValT<MIXED>* __restrict__ v, const double* __restrict__ vplain,
                           int64_t len, const double* __restrict__ vscale, double* __restrict__ y)
{
    pdl_wait();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len;
         i += (int64_t)gridDim.x * blockDim.x) {
        double val;
        if constexpr (MIXED) val = (double)v[i].x + (double)v[i].y;
        else val = vplain ? vplain[i] : v[i];
        y[i] = vscale ? val / vscale[i] : val;
    }
}

// S->beta = ||x|| (one block): the scale of the row-wise A^T u
__global__ void __launch_bounds__(kLThreads)
k_beta_norm(const double* __restrict__ x, int64_t n, LsqrState* __restrict__ S)
{
    pdl_wait();
    __shared__ double red[kLThreads / 32];
    double ss = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) ss += x[i] * x[i];
    ss = block_sum(ss, red);
    if (threadIdx.x == 0) S->beta = sqrt(ss);
}

template <bool MIXED>
static void product_impl(const LsqrProblem& P, char trans, const double* x, double* y,
                         const double* vscale, void* work, cudaStream_t st)
{
    using V = ValT<MIXED>;
    LsqrBufs B = carve(P, work);
    LsqrState init{};
    init.ib = 1.0;   // t = A^T u / beta with beta = 1; coef_n = 0: u = A z
    init.beta = 1.0;
    SKL_CUDA(cudaMemcpyAsync(B.S, &init, sizeof(LsqrState), cudaMemcpyHostToDevice, st));
    SKL_CUDA(cudaMemsetAsync(B.uh, 0, P.n * sizeof(double), st));
    SKL_CUDA(cudaMemsetAsync(B.us, 0, P.n * sizeof(V), st));
    const unsigned g = 152 * 8;
    if (trans == 'n') {
        launch_k(k_prod_in<MIXED>, g, 256, 0, st, x, P.d, vscale, (V*)B.z);
        launch_spmv_n<MIXED>(P, B, st);
        launch_k(k_prod_out<MIXED>, g, 256, 0, st, (const V*)B.us, MIXED ? nullptr : B.uh, P.n, nullptr, y);
    } else {
        launch_k(k_prod_in<MIXED>, g, 256, 0, st, x, P.n, nullptr, (V*)B.us);
        launch_k(k_beta_norm, 1, kLThreads, 0, st, x, P.n, B.S);
        SKL_LAUNCHED();
        launch_spmv_t<MIXED>(P, B, st);
        launch_k(k_prod_out<MIXED>, g, 256, 0, st, (const V*)B.t, nullptr, P.r, vscale, y);
    }
    SKL_LAUNCHED();
    SKL_LAUNCHED();
}

void lsqr_product(const LsqrProblem& P, char trans, const double* x, double* y,
                  const double* vscale, void* work, cudaStream_t st)
{
    if (P.precision == SKL_PREC_MIXED) product_impl<true>(P, trans, x, y, vscale, work, st);
    else product_impl<false>(P, trans, x, y, vscale, work, st);
}

// Final assembly x_full[cols[i]] = colscale[cols[i]] * (M y)[i] with FP64
// accumulation (M upcast exactly): one product per solve, so the solution is
// formed at FP64 accuracy even on the mixed path.
template <typename MT>
__global__ void __launch_bounds__(kTriThreads)
k_tri_n_f64acc(const MT* __restrict__ Mr, int64_t ldm, int r, const double* __restrict__ y,
               const int* __restrict__ cols, const double* __restrict__ colscale,
               double* __restrict__ xfull)
{
    pdl_wait();
    __shared__ double red[kTriThreads / 32];
    for (int i = blockIdx.x; i < r; i += gridDim.x) {
        const MT* row = Mr + (int64_t)i * ldm;
        double acc = 0.0;
        for (int j = i + threadIdx.x; j < r; j += blockDim.x) acc = fma((double)row[j], y[j], acc);
        acc = block_sum(acc, red);
        if (threadIdx.x == 0) {
            const int c = cols[i];
            xfull[c] = colscale[c] * acc;
        }
    }
}

// x_full[cols[i]] = colscale[cols[i]] * (M yv)[i] (FP64 output), other entries untouched.
void precond_apply(const LsqrProblem& P, const double* yv, double* xfull, void* scratch,
                   cudaStream_t st)
{
    if (P.r <= 0) return;
    (void)scratch;
    const unsigned g = (unsigned)std::min<int64_t>(P.r, 152 * 16);
    if (P.precision == SKL_PREC_MIXED)
        launch_k(k_tri_n_f64acc<float>, g, kTriThreads, 0, st, (const float*)P.Mrow, P.ldm, (int)P.r, yv,
                                                         P.cols, P.colscale, xfull);
    else
        launch_k(k_tri_n_f64acc<double>, g, kTriThreads, 0, st, (const double*)P.Mrow, P.ldm, (int)P.r, yv,
                                                          P.cols, P.colscale, xfull);
    SKL_LAUNCHED();
}

// ------------------------------------- refinement of the sketch solution --
// One step of iterative refinement of the sketched least-squares solution
// c* = argmin || S (A D P1 M c - b) || (the explicit solution x_s = D P1 M c
// of ls_sparse_spqr, src/ls_sparse_spqr.cpp:144-151, which the reference forms
// from an FP64 factorization):
//     r  = b - A x            (FP64, by the caller / the previous step)
//     g  = D P1^T A^T S^T S r
//     c += M^T g,  x = D P1 M c,  r = b - A x.
// With M from an FP32 factorization of S A D P1 (= Q R + E, ||E|| ~ eps32 ||S A D||)
// each step contracts the error of c by ~eps32 * cond(R), so two or three
// steps bring x_s to FP64 quality; the LSQR that follows then starts from the
// residual the reference starts from.

// h[i] = sum_t sign(i, t) / sqrt(k) * g[row(i, t)]   (S^T g; hidx[i*k+t] = row | sign bit)
__global__ void k_hash_t(const unsigned* __restrict__ hidx, int n, int k, double v,
                         const double* __restrict__ g, double* __restrict__ h)
{
    pdl_wait();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int t = 0; t < k; ++t) {
            const unsigned e = hidx[(int64_t)i * k + t];
            const double sv = (e & 0x80000000u) ? -v : v;
            acc = fma(sv, g[e & 0x7fffffffu], acc);
        }
        h[i] = acc;
    }
}

// t[i] = colscale[c] * sum_{p in column c} A[p] h[row p],  c = cols[i]  (FP64, warp per column)
__global__ void __launch_bounds__(kLThreads)
k_atr_sel(const int* __restrict__ cp, const int* __restrict__ ri, const double* __restrict__ rx,
          const int* __restrict__ cols, const double* __restrict__ colscale, int r,
          const double* __restrict__ h, double* __restrict__ t)
{
    pdl_wait();
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = gw; i < r; i += nw) {
        const int c = cols[i];
        double a0 = 0.0, a1 = 0.0;
        const int p1 = cp[c + 1];
        int p = cp[c] + lane;
        for (; p + 32 < p1; p += 64) {
            a0 = fma(rx[p], h[ri[p]], a0);
            a1 = fma(rx[p + 32], h[ri[p + 32]], a1);
        }
        if (p < p1) a0 = fma(rx[p], h[ri[p]], a0);
        const double acc = warp_sum(a0 + a1);
        if (lane == 0) t[i] = colscale[c] * acc;
    }
}

// dc[j] = sum_{i <= j} M[i][j] t[i]  (Mc column-major, FP64 accumulation)
template <typename MT>
__global__ void __launch_bounds__(kTriThreads)
k_tri_t_f64(const MT* __restrict__ Mc, int64_t ldm, int r, const double* __restrict__ t,
            double* __restrict__ dc)
{
    pdl_wait();
    __shared__ double red[kTriThreads / 32];
    for (int j = blockIdx.x; j < r; j += gridDim.x) {
        const MT* col = Mc + (int64_t)j * ldm;
        double acc = 0.0;
        for (int i = threadIdx.x; i <= j; i += blockDim.x) acc = fma((double)col[i], t[i], acc);
        acc = block_sum(acc, red);
        if (threadIdx.x == 0) dc[j] = acc;
    }
}

// partial sums of squares of x[0..n) per block (fixed order)
__global__ void __launch_bounds__(kLThreads)
k_sumsq(const double* __restrict__ x, int64_t n, double* __restrict__ part)
{
    pdl_wait();
    __shared__ double red[kLThreads / 32];
    double ss = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        ss += x[i] * x[i];
    ss = block_sum(ss, red);
    if (threadIdx.x == 0) part[blockIdx.x] = ss;
}

// c[i] += sgn * dc[i]
__global__ void k_axpy_sign(int n, double sgn, const double* __restrict__ dc, double* __restrict__ c)
{
    pdl_wait();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        c[i] = fma(sgn, dc[i], c[i]);
}

__global__ void __launch_bounds__(kLThreads)
k_residual_csr(const int* __restrict__ rp, const int* __restrict__ ci, const double* __restrict__ cx,
               int n, const double* __restrict__ x, const double* __restrict__ b,
               double* __restrict__ r, double* __restrict__ part);
__global__ void k_sum_parts(const double* __restrict__ part, int np, double* __restrict__ out);

static void vec_norm(const double* x, int64_t n, double* part, double* out, cudaStream_t st)
{
    const int np = 256;
    launch_k(k_sumsq, np, kLThreads, 0, st, x, n, part);
    launch_k(k_sum_parts, 1, kLThreads, 0, st, part, np, out);
    SKL_LAUNCHED();
    SKL_LAUNCHED();
}

void sketch_refine_direction(const LsqrProblem& P, const int* bptr, const unsigned* bent,
                             const unsigned* hidx, int k, int64_t m, const double* rs, double* gm,
                             double* h, double* t, double* dc, double* part, double* norms,
                             cudaStream_t st)
{
    if (P.r <= 0 || P.Ad64 || P.Ad) fail(SKL_ERR_INVALID, "sketch refinement: sparse problems only");
    sketch_rhs(bptr, bent, m, k, rs, gm, st);
    const double v = 1.0 / std::sqrt((double)k);
    launch_k(k_hash_t, (unsigned)std::min<int64_t>((P.n + 255) / 256, 152 * 16), 256, 0, st, 
        hidx, (int)P.n, k, v, gm, h);
    launch_k(k_atr_sel, (unsigned)std::min<int64_t>((P.r * 32 + kLThreads - 1) / kLThreads, 152 * 32), kLThreads, 0, st, P.cp, P.ri, P.rx64, P.cols, P.colscale, (int)P.r, h, t);
    const unsigned g = (unsigned)std::min<int64_t>(P.r, 152 * 16);
    if (P.precision == SKL_PREC_MIXED)
        launch_k(k_tri_t_f64<float>, g, kTriThreads, 0, st, (const float*)P.M, P.ldm, (int)P.r, t, dc);
    else
        launch_k(k_tri_t_f64<double>, g, kTriThreads, 0, st, (const double*)P.M, P.ldm, (int)P.r, t, dc);
    for (int q = 0; q < 3; ++q) SKL_LAUNCHED();
    vec_norm(gm, m, part, norms, st);
    vec_norm(dc, P.r, part + 256, norms + 1, st);
}

void sketch_refine_apply(const LsqrProblem& P, double sgn, const double* dc, double* c,
                         const double* b, double* x, double* rs, double* part, double* rnorm,
                         cudaStream_t st)
{
    launch_k(k_axpy_sign, (unsigned)std::max<int64_t>(1, std::min<int64_t>((P.r + 255) / 256, 152)), 256, 0, st, (int)P.r, sgn, dc, c);
    SKL_LAUNCHED();
    SKL_CUDA(cudaMemsetAsync(x, 0, P.d * sizeof(double), st));
    precond_apply(P, c, x, nullptr, st);
    const int np = 512;
    launch_k(k_residual_csr, np, kLThreads, 0, st, P.rp, P.ci, P.cx64, (int)P.n, x, b, rs, part);
    launch_k(k_sum_parts, 1, kLThreads, 0, st, part, np, rnorm);
    SKL_LAUNCHED();
    SKL_LAUNCHED();
}

// ------------------------------------------------- FP64 residual checks --
// r = b - A x with plain FP64 (CSR rows or dense columns); partial ||r||^2.
__global__ void __launch_bounds__(kLThreads)
k_residual_csr(const int* __restrict__ rp, const int* __restrict__ ci, const double* __restrict__ cx,
               int n, const double* __restrict__ x, const double* __restrict__ b,
               double* __restrict__ r, double* __restrict__ part)
{
    pdl_wait();
    __shared__ double red[kLThreads / 32];
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    double ss = 0.0;
    for (int i = gw; i < n; i += nw) {
        double acc = 0.0;
        for (int p = rp[i] + lane; p < rp[i + 1]; p += 32) acc = fma(cx[p], x[ci[p]], acc);
        acc = warp_sum(acc);
        if (lane == 0) {
            double v = b[i] - acc;
            r[i] = v;
            ss += v * v;
        }
    }
    ss = block_sum(ss, red);
    if (threadIdx.x == 0) part[blockIdx.x] = ss;
}

__global__ void __launch_bounds__(kLThreads)
k_residual_dense(const double* __restrict__ A, int64_t lda, int n, int d,
                 const double* __restrict__ x, const double* __restrict__ b,
                 double* __restrict__ r, double* __restrict__ part)
{
    pdl_wait();
    __shared__ double red[kLThreads / 32];
    double ss = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int j = 0; j < d; ++j) acc = fma(A[i + (int64_t)j * lda], x[j], acc);
        double v = b[i] - acc;
        r[i] = v;
        ss += v * v;
    }
    ss = block_sum(ss, red);
    if (threadIdx.x == 0) part[blockIdx.x] = ss;
}

// g = A^T r over all d columns, partial ||g||^2
__global__ void __launch_bounds__(kLThreads)
k_atr_csc(const int* __restrict__ cp, const int* __restrict__ ri, const double* __restrict__ rx,
          int d, const double* __restrict__ r, double* __restrict__ part)
{
    pdl_wait();
    __shared__ double red[kLThreads / 32];
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    double ss = 0.0;
    for (int j = gw; j < d; j += nw) {
        double acc = 0.0;
        for (int p = cp[j] + lane; p < cp[j + 1]; p += 32) acc = fma(rx[p], r[ri[p]], acc);
        acc = warp_sum(acc);
        if (lane == 0) ss += acc * acc;
    }
    ss = block_sum(ss, red);
    if (threadIdx.x == 0) part[blockIdx.x] = ss;
}

__global__ void __launch_bounds__(kLThreads)
k_atr_dense(const double* __restrict__ A, int64_t lda, int n, int d, const double* __restrict__ r,
            double* __restrict__ part)
{
    pdl_wait();
    __shared__ double red[kLThreads / 32];
    double ss = 0.0;
    for (int j = blockIdx.x; j < d; j += gridDim.x) {
        double acc = 0.0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) acc = fma(A[i + (int64_t)j * lda], r[i], acc);
        acc = block_sum(acc, red);
        ss += acc * acc;
    }
    if (threadIdx.x == 0) part[blockIdx.x] = ss;
}

__global__ void k_sum_parts(const double* __restrict__ part, int np, double* __restrict__ out)
{
    pdl_wait();
    __shared__ double red[kLThreads / 32];
    double s = 0.0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) s += part[i];
    s = block_sum(s, red);
    if (threadIdx.x == 0) *out = sqrt(s);
}

// out[0] = ||b - A x||, out[1] = ||A^T (b - A x)||; FP64 throughout.
void residual_and_backward(const LsqrProblem& P, const double* x, const double* b, double* r,
                           double* part, double* out, cudaStream_t st)
{
    const int np = 512;
    if (P.Ad64) {
        launch_k(k_residual_dense, np, kLThreads, 0, st, P.Ad64, P.lda64, (int)P.n, (int)P.d, x, b, r, part);
        launch_k(k_sum_parts, 1, kLThreads, 0, st, part, np, out);
        launch_k(k_atr_dense, np, kLThreads, 0, st, P.Ad64, P.lda64, (int)P.n, (int)P.d, r, part);
        launch_k(k_sum_parts, 1, kLThreads, 0, st, part, np, out + 1);
    } else {
        launch_k(k_residual_csr, np, kLThreads, 0, st, P.rp, P.ci, P.cx64, (int)P.n, x, b, r, part);
        launch_k(k_sum_parts, 1, kLThreads, 0, st, part, np, out);
        launch_k(k_atr_csc, np, kLThreads, 0, st, P.cp, P.ri, P.rx64, (int)P.d, r, part);
        launch_k(k_sum_parts, 1, kLThreads, 0, st, part, np, out + 1);
    }
    for (int q = 0; q < 4; ++q) SKL_LAUNCHED();
}

// (hi, lo) float pairs of the equilibrated values A(:, c) * colscale[c] (the
// matrix storage of the mixed sparse path).  The pair carries 48 of the 53
// significand bits (|v - hi - lo| <= 2^-48 |v|); with |v| <= 1 neither part
// overflows, and a value that underflows is below 2^-126 of its column's norm.
__global__ void k_split_csr_scaled(const int* __restrict__ ci, const double* __restrict__ cx,
                                   int64_t nnz, const double* __restrict__ colscale,
                                   float2* __restrict__ out)
{
    pdl_wait();
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nnz;
         p += (int64_t)gridDim.x * blockDim.x) {
        ff f = ff_from_double(cx[p] * colscale[ci[p]]);
        out[p] = make_float2(f.hi, f.lo);
    }
}

void split_csr_scaled(const int* ci, const double* cx, int64_t nnz, const double* colscale,
                      float2* out, cudaStream_t st)
{
    if (nnz <= 0) return;
    unsigned g = (unsigned)std::min<int64_t>((nnz + 255) / 256, 152 * 32);
    launch_k(k_split_csr_scaled, g, 256, 0, st, ci, cx, nnz, colscale, out);
    SKL_LAUNCHED();
}

// CSC variant: one warp per column.
__global__ void __launch_bounds__(kLThreads)
k_split_csc_scaled(const int* __restrict__ cp, const double* __restrict__ Ax, int d,
                   const double* __restrict__ colscale, float2* __restrict__ out)
{
    pdl_wait();
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int c = gw; c < d; c += nw) {
        const double s = colscale[c];
        for (int p = cp[c] + lane; p < cp[c + 1]; p += 32) {
            ff f = ff_from_double(Ax[p] * s);
            out[p] = make_float2(f.hi, f.lo);
        }
    }
}

void split_csc_scaled(const int* cp, const double* Ax, int64_t d, const double* colscale,
                      float2* out, cudaStream_t st)
{
    if (d <= 0) return;
    unsigned g = (unsigned)std::min<int64_t>((d * 32 + kLThreads - 1) / kLThreads, 152 * 16);
    launch_k(k_split_csc_scaled, g, kLThreads, 0, st, cp, Ax, (int)d, colscale, out);
    SKL_LAUNCHED();
}

// Dense matrix: column-major n x d with lda -> packed n x d float2.  A nonzero
// magnitude outside [2^-100, 2^100] sets kStatusRange: the FP32 sketch and
// the float pairs lose accuracy there, and the caller takes the FP64 path.
__global__ void k_split_dense(const double* __restrict__ A, int64_t lda, int64_t n, int64_t d,
                              float2* __restrict__ out, unsigned* __restrict__ status)
{
    pdl_wait();
    const int64_t total = n * d;
    bool bad = false;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e % n, j = e / n;
        const double a = A[i + j * lda];
        const double aa = fabs(a);
        bad |= (aa > 0x1p100) || (aa != 0.0 && aa < 0x1p-100);
        ff f = ff_from_double(a);
        out[e] = make_float2(f.hi, f.lo);
    }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(status, kStatusRange);
}

void split_dense(const double* A, int64_t lda, int64_t n, int64_t d, float2* out,
                 unsigned* status, cudaStream_t st)
{
    if (n * d <= 0) return;
    launch_k(k_split_dense, 152 * 32, 256, 0, st, A, lda, n, d, out, status);
    SKL_LAUNCHED();
}

__global__ void k_vec_add(double* __restrict__ x, const double* __restrict__ a, int64_t n)
{
    pdl_wait();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        x[i] += a[i];
}

void vec_add(double* x, const double* a, int64_t n, cudaStream_t st)
{
    if (n <= 0) return;
    unsigned g = (unsigned)std::min<int64_t>((n + 255) / 256, 152 * 8);
    launch_k(k_vec_add, g, 256, 0, st, x, a, n);
    SKL_LAUNCHED();
}

template <typename T>
__global__ void k_extend_identity(T* __restrict__ Mc, int64_t ldm, int r, int r2)
{
    pdl_wait();
    for (int j = r + blockIdx.x; j < r2; j += gridDim.x) {
        T* col = Mc + (int64_t)j * ldm;
        for (int i = threadIdx.x; i <= j; i += blockDim.x) col[i] = (i == j) ? T(1) : T(0);
    }
}

template <typename T>
void extend_identity(T* Mc, int64_t ldm, int64_t r, int64_t r2, cudaStream_t st)
{
    if (r2 <= r) return;
    unsigned g = (unsigned)std::min<int64_t>(r2 - r, 152 * 8);
    launch_k(k_extend_identity<T>, g, 256, 0, st, Mc, ldm, (int)r, (int)r2);
    SKL_LAUNCHED();
}
template void extend_identity<float>(float*, int64_t, int64_t, int64_t, cudaStream_t);
template void extend_identity<double>(double*, int64_t, int64_t, int64_t, cudaStream_t);

// Row-major copy of the r x r upper triangle (for the forward triangular product).
template <typename T>
__global__ void k_transpose_upper(const T* __restrict__ Mc, int64_t ldm, int r, T* __restrict__ Mr)
{
    pdl_wait();
    __shared__ T tile[32][33];
    const int bi = blockIdx.x * 32, bj = blockIdx.y * 32;
    if (bi > bj + 31) return;   // tile entirely below the diagonal
    for (int q = threadIdx.y; q < 32; q += blockDim.y) {
        int i = bi + threadIdx.x, j = bj + q;
        tile[q][threadIdx.x] = (i < r && j < r) ? Mc[i + (int64_t)j * ldm] : T(0);
    }
    __syncthreads();
    for (int q = threadIdx.y; q < 32; q += blockDim.y) {
        int j = bj + threadIdx.x, i = bi + q;
        if (i < r && j < r) Mr[j + (int64_t)i * ldm] = tile[threadIdx.x][q];
    }
}

template <typename T>
void transpose_upper(const T* Mc, int64_t ldm, int64_t r, T* Mr, cudaStream_t st)
{
    if (r <= 0) return;
    dim3 g((unsigned)((r + 31) / 32), (unsigned)((r + 31) / 32));
    launch_k(k_transpose_upper<T>, g, dim3(32, 8), 0, st, Mc, ldm, (int)r, Mr);
    SKL_LAUNCHED();
}
template void transpose_upper<float>(const float*, int64_t, int64_t, float*, cudaStream_t);
template void transpose_upper<double>(const double*, int64_t, int64_t, double*, cudaStream_t);

}  // namespace skl
