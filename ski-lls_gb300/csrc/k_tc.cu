// k_tc.cu -- tensor-core (tcgen05) products of the randomized CPQR, sm_103a.
//
// W = V^T A for the block reflector of one panel (the first product of
// dlarfb in HQRRP's trailing update, hqrrp/.../NoFLA_HQRRP_WY_blk_var4_skint.c:
// 547-550): V is the M x b panel of Householder vectors (b <= 64), A the
// M x N trailing matrix, W is b x N.  FP32 data, 3xTF32 arithmetic on the
// 5th-generation tensor cores:  a = hi(a) + lo(a) with hi = a rounded to the
// nearest TF32 value and lo = a - hi rounded to the nearest TF32 value, and
//     V^T A ~ hi(V)^T hi(A) + lo(V)^T hi(A) + hi(V)^T lo(A)
// accumulated in FP32 in tensor memory (each product within ~2^-24 of its
// magnitude, like an FP32 FMA: the dropped lo*lo term and lo's own rounding
// are each at most 2^-24).
//
// One CTA owns 128 columns of A and a range of K (rows of A and V); the MMA
// computes D[128 x 64] = A_tile^T V_tile (M = 128 columns of A, N = 64
// reflectors, K = 8 per instruction), so both operands are K-major in shared
// memory with the 128-byte swizzle the TMA writes.  Warp roles:
//   warp 0     TMA producer: A tile (32 rows x 128 columns) and the pre-split
//              V hi / lo tiles (32 rows x 64 columns) per stage
//   warp 1     TMEM allocation; one thread issues the 12 MMAs of a stage and
//              commits them to the stage's "empty" barrier
//   warps 2-5  split each A tile into hi (in place) and lo
//   warps 6-13 every kGroup stages, read the accumulator out of TMEM (each
//              warp 32 reflectors of its 32-lane quadrant) into Kahan-
//              compensated register sums, and at the end write the CTA's
//              partial W
// Split-K partials are summed by a fixed-order reduction, so W is bitwise
// reproducible.  Every mbarrier wait is bounded: a wait that gives up sets
// kStatusTcTimeout in the status word, the CTA stops issuing work, waits
// (bounded) for its own copies and MMAs, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "skl_internal.hpp"
#include "launch.cuh"
#include "common.cuh"
#include "k_gemm.cuh"

namespace skl {

namespace {

constexpr int kTcThreads = 448;   // producer, MMA, 4 converter and 8 drainer warps
constexpr int kBK = 32;          // K rows per stage: 32 FP32 = one 128-byte swizzle row
constexpr int kTM = 128;         // A columns per CTA (MMA M)
constexpr int kTN = 64;          // reflectors (MMA N)
constexpr int kStages = 4;
constexpr int kABytes = kTM * kBK * 4;    // 16 KB
constexpr int kVBytes = kTN * kBK * 4;    // 8 KB
// stage: A hi (TMA'd raw, split in place), A lo, V hi, V lo
constexpr int kStageBytes = 2 * kABytes + 2 * kVBytes;
constexpr int kTxBytes = kABytes + 2 * kVBytes;   // bytes the TMA delivers per stage
constexpr int kSmemBytes = kStages * kStageBytes + 1024 /* barriers */ + 1024 /* alignment */;
constexpr int kGroup = 2;        // stages accumulated in TMEM before a drain
constexpr unsigned kTmemCols = 128;   // two 64-column accumulators
constexpr unsigned kWaitLimit = 1u << 22;

// ---- PTX wrappers -------------------------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void* p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(unsigned bar)
{
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes)
{
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(bar),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try(unsigned bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for the phase with the given parity; false (and the status
// bit) when the limit is reached.
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity, unsigned* status)
{
    for (unsigned i = 0; i < kWaitLimit; ++i)
        if (mbar_try(bar, parity)) return true;
    atomicOr(status, kStatusTcTimeout);
    return false;
}

__device__ __forceinline__ void tma_load_2d(unsigned dst, const CUtensorMap* map, int x, int y,
                                            unsigned bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (SBO), tile base 1024-byte aligned.
__device__ __forceinline__ uint64_t sw128_desc(unsigned addr)
{
    uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;              // LBO (unused by swizzled K-major layouts)
    d |= (uint64_t)(1024 >> 4) << 32;    // SBO
    d |= (uint64_t)1 << 46;              // descriptor version (tcgen05)
    d |= (uint64_t)2 << 61;              // SWIZZLE_128B
    return d;
}

// Instruction descriptor, kind::tf32: D FP32, A and B TF32, both K-major.
__host__ __device__ constexpr uint32_t tf32_idesc(int M, int N)
{
    return (1u << 4)                       // D format F32
         | (2u << 7) | (2u << 10)          // A, B format TF32
         | ((uint32_t)(N >> 3) << 17)
         | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(unsigned d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         unsigned accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mma_commit(unsigned bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

// 32 consecutive TMEM columns of this warp's lane quadrant.
__device__ __forceinline__ void tmem_ld32(unsigned taddr, float (&v)[32])
{
    unsigned r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
        "%13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
          "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
          "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
          "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int q = 0; q < 32; ++q) v[q] = __uint_as_float(r[q]);
}

// a rounded to the nearest TF32 value (low 13 significand bits zero).  The
// splits are hi = rna(a) and lo = rna(a - hi): both exact TF32 operands, with
// |a - hi - lo| <= 2^-24 |a|, so the three products carry ~2^-24 per term.
__device__ __forceinline__ float tf32_hi(float a)
{
    unsigned r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(a));
    return __uint_as_float(r);
}

// ---- W = V^T A -------------------------------------------------------------
// Grid (column tiles, K splits).  partial: W of split z at partial + z*b*N
// (b x N, column-major, ld b).
//
// The tensor core's FP32 accumulator rounds at every MMA; summed over a
// CTA's whole K range (up to ~800 accumulations of a 3xTF32 product) that
// left W ~1.6e-6 off (normwise) at K = 8,500, ten times the CUDA-core FP32
// kernel, which lifted an FP32 pivoted factorization's noise floor for
// dependent columns from 7e-7 to 1.6e-5 of |R_00|.  So the accumulator lives
// for only kGroup stages (64 rows of K): drainer warps read it out of tensor
// memory (double-buffered, so the MMAs of the next group proceed) and add it
// into registers with Kahan compensation.
__global__ void __launch_bounds__(kTcThreads, 1)
k_tc_vta(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapVh,
         const __grid_constant__ CUtensorMap mapVl, int N, int b, int kb_per, int kb_total,
         float* __restrict__ partial, unsigned* __restrict__ status)
{
    pdl_wait();
    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + kStages * kStageBytes);
    // bars: full[kStages], conv[kStages], empty[kStages], tfull[2], tempty[2], done;
    // then the TMEM address
    unsigned* tmem_slot = reinterpret_cast<unsigned*>(bars + 3 * kStages + 5);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int col0 = blockIdx.x * kTM;
    const int kb0 = blockIdx.y * kb_per;
    const int nkb = min(kb_per, kb_total - kb0);
    const int ngroups = (nkb + kGroup - 1) / kGroup;
    auto full = [&](int s) { return smem_u32(bars + s); };
    auto conv = [&](int s) { return smem_u32(bars + kStages + s); };
    auto empty = [&](int s) { return smem_u32(bars + 2 * kStages + s); };
    auto tfull = [&](int q) { return smem_u32(bars + 3 * kStages + q); };
    auto tempty = [&](int q) { return smem_u32(bars + 3 * kStages + 2 + q); };
    const unsigned done = smem_u32(bars + 3 * kStages + 4);
    auto a_hi = [&](int s) { return smem + s * kStageBytes; };
    auto a_lo = [&](int s) { return smem + s * kStageBytes + kABytes; };
    auto v_hi = [&](int s) { return smem + s * kStageBytes + 2 * kABytes; };
    auto v_lo = [&](int s) { return smem + s * kStageBytes + 2 * kABytes + kVBytes; };

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(full(s), 1);
            mbar_init(conv(s), 128);
            mbar_init(empty(s), 1);
        }
        for (int q = 0; q < 2; ++q) {
            mbar_init(tfull(q), 1);
            mbar_init(tempty(q), 256);
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mapA)) : "memory");
            bool ok = true;
            int issued = 0;
            for (int kb = 0; kb < nkb && ok; ++kb) {
                const int s = kb % kStages;
                if (kb >= kStages) ok = mbar_wait(empty(s), ((kb / kStages) - 1) & 1, status);
                if (!ok) break;
                mbar_expect_tx(full(s), kTxBytes);
                const int krow = (kb0 + kb) * kBK;
                tma_load_2d(smem_u32(a_hi(s)), &mapA, krow, col0, full(s));
                tma_load_2d(smem_u32(v_hi(s)), &mapVh, krow, 0, full(s));
                tma_load_2d(smem_u32(v_lo(s)), &mapVl, krow, 0, full(s));
                ++issued;
            }
            // the copies this CTA issued have landed before it may exit
            for (int kb = std::max(0, issued - kStages); kb < issued; ++kb)
                mbar_wait(full(kb % kStages), (kb / kStages) & 1, status);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = tf32_idesc(kTM, kTN);
            bool ok = true;
            for (int kb = 0; kb < nkb && ok; ++kb) {
                const int s = kb % kStages;
                const int g = kb / kGroup, buf = g & 1;
                const bool first = (kb % kGroup) == 0;
                if (first && g >= 2) ok = mbar_wait(tempty(buf), ((g >> 1) - 1) & 1, status);
                if (ok) ok = mbar_wait(conv(s), (kb / kStages) & 1, status);
                if (!ok) break;
                tc_fence_after();
                const unsigned d = tmem + (unsigned)(buf * kTN);
                const unsigned ah = smem_u32(a_hi(s)), al = smem_u32(a_lo(s));
                const unsigned vh = smem_u32(v_hi(s)), vl = smem_u32(v_lo(s));
#pragma unroll
                for (int k8 = 0; k8 < kBK / 8; ++k8) {
                    const unsigned off = k8 * 32;   // 8 TF32 values along K
                    mma_tf32(d, sw128_desc(al + off), sw128_desc(vh + off), idesc,
                             (first && k8 == 0) ? 0u : 1u);
                    mma_tf32(d, sw128_desc(ah + off), sw128_desc(vl + off), idesc, 1u);
                    mma_tf32(d, sw128_desc(ah + off), sw128_desc(vh + off), idesc, 1u);
                }
                mma_commit(empty(s));
                if ((kb % kGroup) == kGroup - 1 || kb == nkb - 1) mma_commit(tfull(buf));
            }
            // every MMA issued here has completed before the TMEM is freed
            mma_commit(done);
            mbar_wait(done, 0, status);
        }
    } else if (warp < 6) {
        // warps 2..5: split A tiles into hi / lo
        const int t = threadIdx.x - 64;
        for (int kb = 0; kb < nkb; ++kb) {
            const int s = kb % kStages;
            if (!mbar_wait(full(s), (kb / kStages) & 1, status)) break;
            float4* h = reinterpret_cast<float4*>(a_hi(s));
            float4* l = reinterpret_cast<float4*>(a_lo(s));
#pragma unroll
            for (int q = 0; q < kABytes / 16 / 128; ++q) {
                const int e = t + q * 128;
                const float4 v = h[e];
                float4 hi, lo;
                hi.x = tf32_hi(v.x); lo.x = tf32_hi(v.x - hi.x);
                hi.y = tf32_hi(v.y); lo.y = tf32_hi(v.y - hi.y);
                hi.z = tf32_hi(v.z); lo.z = tf32_hi(v.z - hi.z);
                hi.w = tf32_hi(v.w); lo.w = tf32_hi(v.w - hi.w);
                h[e] = hi;
                l[e] = lo;
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_arrive(conv(s));
        }
    } else {
        // warps 6..13: drain each group's accumulator into Kahan sums; this
        // warp's 32-lane quadrant = 32 columns of A, `half` = which 32 of the
        // 64 reflectors
        const int quad = warp & 3;
        const int half = (warp - 6) >> 2;
        float sum[32], comp[32];
#pragma unroll
        for (int q = 0; q < 32; ++q) sum[q] = comp[q] = 0.f;
        bool ok = true;
        for (int g = 0; g < ngroups; ++g) {
            const int buf = g & 1;
            ok = __all_sync(0xffffffffu, mbar_wait(tfull(buf), (g >> 1) & 1, status));
            if (!ok) break;   // warp-uniform: tcgen05.ld is warp-collective
            tc_fence_after();
            {
                float v[32];
                tmem_ld32(tmem + ((unsigned)(quad * 32) << 16) + (unsigned)(buf * kTN + half * 32), v);
#pragma unroll
                for (int q = 0; q < 32; ++q) {
                    const float y = __fsub_rn(v[q], comp[q]);
                    const float t2 = __fadd_rn(sum[q], y);
                    comp[q] = __fsub_rn(__fsub_rn(t2, sum[q]), y);
                    sum[q] = t2;
                }
            }
            tc_fence_before();
            mbar_arrive(tempty(buf));
        }
        const int col = col0 + quad * 32 + lane;
        if (ok && nkb > 0 && col < N) {
            float* out = partial + (int64_t)blockIdx.y * b * N + (int64_t)col * b + half * 32;
            if (b == kTN) {
#pragma unroll
                for (int q = 0; q < 32; q += 4)
                    *reinterpret_cast<float4*>(out + q) = make_float4(sum[q], sum[q + 1], sum[q + 2], sum[q + 3]);
            } else {
#pragma unroll
                for (int q = 0; q < 32; ++q)
                    if (half * 32 + q < b) out[q] = sum[q];
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols)
                     : "memory");
    }
}

// V (M x b, ldv) -> hi / lo (M x b, ldvs)
__global__ void k_tc_split_v(const float* __restrict__ V, int64_t ldv, int M, int b,
                             float* __restrict__ Vh, float* __restrict__ Vl, int64_t ldvs)
{
    pdl_wait();
    const int64_t total = (int64_t)M * b;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % M), c = (int)(e / M);
        const float a = V[i + (int64_t)c * ldv];
        const float h = tf32_hi(a);
        Vh[i + (int64_t)c * ldvs] = h;
        Vl[i + (int64_t)c * ldvs] = tf32_hi(a - h);
    }
}

// ---- C -= V Z (the trailing update) ------------------------------------------
// C is the M x N trailing block (column-major, ld), V the panel's M x b
// reflectors, Z = T^T W (b x N).  Rows r0.. of C are updated (the first b
// rows, R12, go ahead as their own small product).  D[128 x 64] = Vt_tile Zt_tile
// with M = 128 rows of C, N = 64 columns, K = b <= 64 (both operands K-major:
// Vt is V stored row by row, Zt is Z with leading dimension 64), 3xTF32.
// One CTA owns a 128-row tile (its V hi / lo stay in shared memory) and a
// run of 64-column tiles: Z tiles through a 2-stage ring, C tiles TMA-loaded
// into a 3-stage ring, updated in place by the epilogue warps from the TMEM
// accumulator (double-buffered), and TMA-stored back.
constexpr int kUpdThreads = 192;   // producer, MMA, 4 epilogue warps
constexpr int kUN = 64;            // columns per tile (MMA N)
constexpr int kUZStages = 2;
constexpr int kUCStages = 3;
constexpr int kUVBytes = 4 * kTM * kBK * 4;          // hi/lo x 2 K halves x 128 rows x 128 B
constexpr int kUZBytes = 4 * kUN * kBK * 4;          // hi/lo x 2 K halves x 64 rows x 128 B
constexpr int kUCBytes = kTM * kUN * 4;              // 128 rows x 64 columns
constexpr int kUSmemBytes = kUVBytes + kUZStages * kUZBytes + kUCStages * kUCBytes + 1024 + 1024;
constexpr unsigned kUTmemCols = 2 * kUN;

__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, int x, int y, unsigned src)
{
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                     reinterpret_cast<uint64_t>(map)),
                 "r"(x), "r"(y), "r"(src)
                 : "memory");
}

__global__ void __launch_bounds__(kUpdThreads, 1)
k_tc_update(const __grid_constant__ CUtensorMap mapVh, const __grid_constant__ CUtensorMap mapVl,
            const __grid_constant__ CUtensorMap mapZh, const __grid_constant__ CUtensorMap mapZl,
            const __grid_constant__ CUtensorMap mapC, int r0, int nct, int ct_per,
            unsigned* __restrict__ status)
{
    pdl_wait();
    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char* vbuf = smem;                                   // [hi0, hi1, lo0, lo1] x 16 KB
    unsigned char* zbuf = smem + kUVBytes;                        // [stage][hi0, hi1, lo0, lo1] x 8 KB
    unsigned char* cbuf = zbuf + kUZStages * kUZBytes;            // [stage] 128 x 64 floats
    uint64_t* bars = reinterpret_cast<uint64_t*>(cbuf + kUCStages * kUCBytes);
    // vfull, zfull[2], zempty[2], cfull[3], cempty[3], tfull[2], tempty[2], done
    unsigned* tmem_slot = reinterpret_cast<unsigned*>(bars + 16);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row = r0 + blockIdx.x * kTM;            // first row of C of this CTA
    const int ct0 = blockIdx.y * ct_per;
    const int nt = min(ct_per, nct - ct0);
    const unsigned vfull = smem_u32(bars + 0);
    auto zfull = [&](int q) { return smem_u32(bars + 1 + q); };
    auto zempty = [&](int q) { return smem_u32(bars + 3 + q); };
    auto cfull = [&](int q) { return smem_u32(bars + 5 + q); };
    auto cempty = [&](int q) { return smem_u32(bars + 8 + q); };
    auto tfull = [&](int q) { return smem_u32(bars + 11 + q); };
    auto tempty = [&](int q) { return smem_u32(bars + 13 + q); };
    const unsigned done = smem_u32(bars + 15);
    auto vtile = [&](int part) { return vbuf + part * (kTM * kBK * 4); };          // part = 2*lo + khalf
    auto ztile = [&](int st, int part) { return zbuf + st * kUZBytes + part * (kUN * kBK * 4); };
    auto ctile = [&](int st) { return cbuf + st * kUCBytes; };

    if (threadIdx.x == 0) {
        mbar_init(vfull, 1);
        for (int q = 0; q < kUZStages; ++q) {
            mbar_init(zfull(q), 1);
            mbar_init(zempty(q), 1);
        }
        for (int q = 0; q < kUCStages; ++q) {
            mbar_init(cfull(q), 1);
            mbar_init(cempty(q), 1);
        }
        for (int q = 0; q < 2; ++q) {
            mbar_init(tfull(q), 1);
            mbar_init(tempty(q), 128);
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(kUTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            bool ok = true;
            mbar_expect_tx(vfull, kUVBytes);
            for (int part = 0; part < 4; ++part)
                tma_load_2d(smem_u32(vtile(part)), (part >> 1) ? &mapVl : &mapVh, (part & 1) * kBK, row,
                            vfull);
            int zi = 0, ci = 0;
            for (int t = 0; t < nt && ok; ++t) {
                const int col = (ct0 + t) * kUN;
                const int zs = t % kUZStages, cs = t % kUCStages;
                if (t >= kUZStages) ok = mbar_wait(zempty(zs), ((t / kUZStages) - 1) & 1, status);
                if (!ok) break;
                mbar_expect_tx(zfull(zs), kUZBytes);
                for (int part = 0; part < 4; ++part)
                    tma_load_2d(smem_u32(ztile(zs, part)), (part >> 1) ? &mapZl : &mapZh, (part & 1) * kBK,
                                col, zfull(zs));
                ++zi;
                if (t >= kUCStages) ok = mbar_wait(cempty(cs), ((t / kUCStages) - 1) & 1, status);
                if (!ok) break;
                mbar_expect_tx(cfull(cs), kUCBytes);
                tma_load_2d(smem_u32(ctile(cs)), &mapC, row, col, cfull(cs));
                ++ci;
            }
            // this CTA's copies have landed before it may exit
            mbar_wait(vfull, 0, status);
            for (int t = std::max(0, zi - kUZStages); t < zi; ++t)
                mbar_wait(zfull(t % kUZStages), (t / kUZStages) & 1, status);
            for (int t = std::max(0, ci - kUCStages); t < ci; ++t)
                mbar_wait(cfull(t % kUCStages), (t / kUCStages) & 1, status);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = tf32_idesc(kTM, kUN);
            bool ok = mbar_wait(vfull, 0, status);
            for (int t = 0; t < nt && ok; ++t) {
                const int zs = t % kUZStages, tb = t & 1;
                ok = mbar_wait(zfull(zs), (t / kUZStages) & 1, status);
                if (ok && t >= 2) ok = mbar_wait(tempty(tb), ((t >> 1) - 1) & 1, status);
                if (!ok) break;
                tc_fence_after();
                const unsigned d = tmem + (unsigned)(tb * kUN);
#pragma unroll
                for (int k8 = 0; k8 < 2 * kBK / 8; ++k8) {
                    const int kh = k8 >> 2;
                    const unsigned off = (k8 & 3) * 32;
                    const unsigned ah = smem_u32(vtile(kh)) + off, al = smem_u32(vtile(2 + kh)) + off;
                    const unsigned bh = smem_u32(ztile(zs, kh)) + off, bl = smem_u32(ztile(zs, 2 + kh)) + off;
                    mma_tf32(d, sw128_desc(al), sw128_desc(bh), idesc, k8 > 0 ? 1u : 0u);
                    mma_tf32(d, sw128_desc(ah), sw128_desc(bl), idesc, 1u);
                    mma_tf32(d, sw128_desc(ah), sw128_desc(bh), idesc, 1u);
                }
                mma_commit(zempty(zs));
                mma_commit(tfull(tb));
            }
            mma_commit(done);
            mbar_wait(done, 0, status);
        }
    } else {
        // warps 2..5: C tile -= D, each thread one row of the tile
        const int quad = warp & 3;
        const int r = quad * 32 + lane;
        const bool leader = threadIdx.x == 64;
        volatile int* s_fail = reinterpret_cast<volatile int*>(tmem_slot + 1);
        if (leader) *s_fail = 0;
        asm volatile("bar.sync 1, 128;" ::: "memory");
        int stored = 0;
        for (int t = 0; t < nt; ++t) {
            const int tb = t & 1, cs = t % kUCStages;
            const bool got = mbar_wait(tfull(tb), (t >> 1) & 1, status) &&
                             mbar_wait(cfull(cs), (t / kUCStages) & 1, status);
            // the four warps leave together: the named barriers below have no timeout
            if (!got) *s_fail = 1;
            asm volatile("bar.sync 1, 128;" ::: "memory");
            if (*s_fail) break;
            tc_fence_after();
            float* c = reinterpret_cast<float*>(ctile(cs));
#pragma unroll
            for (int h = 0; h < kUN / 32; ++h) {
                float v[32];
                tmem_ld32(tmem + ((unsigned)(quad * 32) << 16) + (unsigned)(tb * kUN + h * 32), v);
#pragma unroll
                for (int q = 0; q < 32; ++q) c[(h * 32 + q) * kTM + r] -= v[q];
            }
            tc_fence_before();
            mbar_arrive(tempty(tb));
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("bar.sync 1, 128;" ::: "memory");
            if (leader) {
                tma_store_2d(&mapC, row, (ct0 + t) * kUN, smem_u32(c));
                asm volatile("cp.async.bulk.commit_group;" ::: "memory");
                ++stored;
                // the previous tile's store has read its stage: release it
                asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
                if (t >= 1) mbar_arrive(cempty((t - 1) % kUCStages));
            }
        }
        if (leader && stored > 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        __syncwarp();
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kUTmemCols)
                     : "memory");
    }
}

// Vt (rows of V, ld 64) and Zt (Z with ld 64) split into hi / lo
__global__ void k_tc_split_vz(const float* __restrict__ V, int64_t ldv, int M, int b,
                              const float* __restrict__ Z, int64_t ldz, int N, float* __restrict__ Vth,
                              float* __restrict__ Vtl, float* __restrict__ Zth, float* __restrict__ Ztl)
{
    pdl_wait();
    const int64_t nv = (int64_t)M * b, total = nv + (int64_t)N * b;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        if (e < nv) {
            const int c = (int)(e % b), i = (int)(e / b);
            const float a = V[i + (int64_t)c * ldv];
            const float h = tf32_hi(a);
            Vth[(int64_t)i * kTN + c] = h;
            Vtl[(int64_t)i * kTN + c] = tf32_hi(a - h);
        } else {
            const int64_t f = e - nv;
            const int c = (int)(f % b), n = (int)(f / b);
            const float a = Z[c + (int64_t)n * ldz];
            const float h = tf32_hi(a);
            Zth[c + (int64_t)n * kTN] = h;
            Ztl[c + (int64_t)n * kTN] = tf32_hi(a - h);
        }
    }
}

// ---- host side ---------------------------------------------------------------
using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*,
                                 CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                 CUtensorMapFloatOOBfill);

EncodeTiled encode_fn()
{
    static EncodeTiled fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
        cudaGetLastError();
    });
    if (!fn) fail(SKL_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    return fn;
}

// 2-D FP32 tensor map over a column-major matrix (rows x cols, ld elements),
// box {32 rows, box_cols}, 128-byte swizzle, zero fill outside.
CUtensorMap map_f32(const float* base, int64_t rows, int64_t cols, int64_t ld, int box_cols)
{
    if (((uintptr_t)base & 15) || ((ld * 4) & 15))
        fail(SKL_ERR_INVALID, "tensor map: base or stride not 16-byte aligned");
    CUtensorMap m;
    cuuint64_t dims[2] = {(cuuint64_t)rows, (cuuint64_t)cols};
    cuuint64_t strides[1] = {(cuuint64_t)(ld * 4)};
    cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_cols};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)base, dims, strides, box, estr,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) fail(SKL_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return m;
}

int sm_count()
{
    static int v = [] {
        int dev = 0, n = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        return n > 0 ? n : 148;
    }();
    return v;
}

}  // namespace

size_t tc_vta_scratch_floats(int64_t M)
{
    const int64_t ldvs = (M + 31) / 32 * 32;
    // V hi / lo, and the split-K partials: splits <= SMs / column tiles, so
    // splits * b * N <= SMs * 64 * 128
    return (size_t)(2 * ldvs * kTN) + (size_t)kTN * kTM * sm_count();
}

void tc_vta(int M, int N, int b, const float* V, int64_t ldv, const float* A, int64_t lda, float* W,
            float* scratch, size_t scratch_floats, unsigned* status, cudaStream_t st)
{
    if (M <= 0 || N <= 0 || b <= 0) return;
    if (b > kTN) fail(SKL_ERR_INVALID, "tc_vta: panel wider than 64");
    const int64_t ldvs = (int64_t)(M + 31) / 32 * 32;
    float* Vh = scratch;
    float* Vl = scratch + ldvs * kTN;
    float* partial = scratch + 2 * ldvs * kTN;
    const int64_t part_cap = (int64_t)scratch_floats - 2 * ldvs * kTN;
    {
        const int64_t total = (int64_t)M * b;
        const unsigned g = (unsigned)std::min<int64_t>((total + 255) / 256, 152 * 8);
        launch_k(k_tc_split_v, g, 256, 0, st, V, ldv, M, b, Vh, Vl, ldvs);
        SKL_LAUNCHED();
    }
    const int ntile = (N + kTM - 1) / kTM;
    const int kb_total = (M + kBK - 1) / kBK;
    // one wave: at most one CTA per SM (each holds ~197 KB of shared memory)
    int splits = std::max(1, std::min(sm_count() / ntile, kb_total / 4));
    while (splits > 1 && (int64_t)splits * b * N > part_cap) --splits;
    const int kb_per = (kb_total + splits - 1) / splits;
    splits = (kb_total + kb_per - 1) / kb_per;
    float* out = splits > 1 ? partial : W;
    const CUtensorMap mA = map_f32(A, M, N, lda, kTM);
    const CUtensorMap mVh = map_f32(Vh, M, b, ldvs, kTN);
    const CUtensorMap mVl = map_f32(Vl, M, b, ldvs, kTN);
    static std::once_flag attr_once;
    std::call_once(attr_once, [] {
        cudaFuncSetAttribute((const void*)k_tc_vta, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
    });
    launch_k(k_tc_vta, dim3(ntile, splits), kTcThreads, kSmemBytes, st, mA, mVh, mVl, N, b, kb_per, kb_total,
                                                                out, status);
    SKL_LAUNCHED();
    if (splits > 1) splitk_reduce_launch<float>(b, N, splits, 1.0f, partial, 0.0f, W, b, st);
}

size_t tc_update_scratch_floats(int64_t M, int64_t N)
{
    return (size_t)(2 * M * kTN + 2 * N * kTN) + 64;
}

void tc_update(int M, int N, int b, int r0, const float* V, int64_t ldv, const float* Z, int64_t ldz,
               float* C, int64_t ldc, float* scratch, unsigned* status, cudaStream_t st)
{
    if (M - r0 <= 0 || N <= 0 || b <= 0) return;
    if (b > kTN) fail(SKL_ERR_INVALID, "tc_update: panel wider than 64");
    float* Vth = scratch;
    float* Vtl = Vth + (int64_t)M * kTN;
    float* Zth = Vtl + (int64_t)M * kTN;
    float* Ztl = Zth + (int64_t)N * kTN;
    {
        const int64_t total = (int64_t)(M + N) * b;
        const unsigned g = (unsigned)std::min<int64_t>((total + 255) / 256, 152 * 8);
        launch_k(k_tc_split_vz, g, 256, 0, st, V, ldv, M, b, Z, ldz, N, Vth, Vtl, Zth, Ztl);
        SKL_LAUNCHED();
    }
    // K-major operands: dims {K = b, rows}, rows 64 floats apart; C: {rows, cols}
    auto kmap = [&](const float* base, int64_t rows, int box_rows) {
        CUtensorMap m;
        cuuint64_t dims[2] = {(cuuint64_t)b, (cuuint64_t)rows};
        cuuint64_t strides[1] = {(cuuint64_t)(kTN * 4)};
        cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
        cuuint32_t estr[2] = {1, 1};
        CUresult r = encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)base, dims, strides, box, estr,
                                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                 CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) fail(SKL_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
        return m;
    };
    const CUtensorMap mVh = kmap(Vth, M, kTM), mVl = kmap(Vtl, M, kTM);
    const CUtensorMap mZh = kmap(Zth, N, kUN), mZl = kmap(Ztl, N, kUN);
    CUtensorMap mC;
    {
        if (((uintptr_t)C & 15) || ((ldc * 4) & 15))
            fail(SKL_ERR_INVALID, "tc_update: C base or stride not 16-byte aligned");
        cuuint64_t dims[2] = {(cuuint64_t)M, (cuuint64_t)N};
        cuuint64_t strides[1] = {(cuuint64_t)(ldc * 4)};
        cuuint32_t box[2] = {(cuuint32_t)kTM, (cuuint32_t)kUN};
        cuuint32_t estr[2] = {1, 1};
        CUresult r = encode_fn()(&mC, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, (void*)C, dims, strides, box, estr,
                                 CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                 CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) fail(SKL_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    }
    const int nrt = (M - r0 + kTM - 1) / kTM;
    const int nct = (N + kUN - 1) / kUN;
    int splits = std::max(1, std::min(nct, sm_count() / nrt));
    const int ct_per = (nct + splits - 1) / splits;
    splits = (nct + ct_per - 1) / ct_per;
    static std::once_flag attr_once;
    std::call_once(attr_once, [] {
        cudaFuncSetAttribute((const void*)k_tc_update, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kUSmemBytes);
    });
    launch_k(k_tc_update, dim3(nrt, splits), kUpdThreads, kUSmemBytes, st, mVh, mVl, mZh, mZl, mC, r0, nct, ct_per,
                                                                     status);
    SKL_LAUNCHED();
}

void update_product(bool tensor, int M, int N, int b, int r0, const float* V, int64_t ldv,
                    const float* Z, int64_t ldz, float* C, int64_t ldc, float* scratch,
                    unsigned* status, cudaStream_t st)
{
    if (tensor)
        tc_update(M, N, b, r0, V, ldv, Z, ldz, C, ldc, scratch, status, st);
    else
        gemm<float>(false, false, M - r0, N, b, -1.0f, V + r0, ldv, Z, ldz, 1.0f, C + r0, ldc, nullptr,
                    0, st);
}

bool tc_qr_enabled()
{
    static const bool v = [] {
        const char* e = getenv("SKILLS_QR_TC");
        return !(e && e[0] == '0');
    }();
    return v;
}

void vta_product(bool tensor, int M, int N, int b, const float* V, int64_t ldv, const float* A,
                 int64_t lda, float* W, float* scratch, size_t scratch_floats, unsigned* status,
                 cudaStream_t st)
{
    if (tensor)
        tc_vta(M, N, b, V, ldv, A, lda, W, scratch, scratch_floats, status, st);
    else
        gemm<float>(true, false, b, N, M, 1.0f, V, ldv, A, lda, 0.0f, W, b, scratch,
                    (int64_t)scratch_floats, st);
}

}  // namespace skl
