// common.cuh -- shared device helpers for the Ski-LLS GB300 solver.
//
//  * float-float ("double-FP32") arithmetic.  GB300's FP64 pipe issues about
//    one FP64 FMA for every 67 FP32 FMAs, so the FP64-accurate inner products
//    of the mixed path (SpMV accumulators, application of R^{-1}) are carried
//    as unevaluated sums hi+lo of two floats (error-free transformations of
//    Dekker/Knuth: TwoSum, TwoProd via fmaf).  Relative accuracy ~2^-48.
//  * warp/block reductions, bounded spin waits, status words.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define SKL_DEV __device__ __forceinline__

namespace skl {

constexpr int kWarp = 32;

// ------------------------------------------------------------------ ff ----
struct ff {
    float hi, lo;
};

SKL_DEV ff ff_from_double(double x)
{
    float h = __double2float_rn(x);
    float l = __double2float_rn(x - (double)h);
    return {h, l};
}

SKL_DEV double ff_to_double(ff a) { return (double)a.hi + (double)a.lo; }

// Knuth TwoSum: s + e == a + b exactly.
SKL_DEV void two_sum(float a, float b, float& s, float& e)
{
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// acc += (p_hi + p_lo), renormalised.
SKL_DEV void ff_add(ff& acc, float p_hi, float p_lo)
{
    float s, e;
    two_sum(acc.hi, p_hi, s, e);
    e = __fadd_rn(e, __fadd_rn(acc.lo, p_lo));
    float h = __fadd_rn(s, e);
    acc.lo = __fsub_rn(e, __fsub_rn(h, s));
    acc.hi = h;
}

SKL_DEV void ff_add(ff& acc, ff b) { ff_add(acc, b.hi, b.lo); }

// acc += a * x where a is an exact float and x = x.hi + x.lo.
SKL_DEV void ff_fma_f(ff& acc, float a, ff x)
{
    float p = __fmul_rn(a, x.hi);
    float pe = __fmaf_rn(a, x.hi, -p);       // exact error of a*x.hi
    float pl = __fmaf_rn(a, x.lo, pe);
    ff_add(acc, p, pl);
}

// acc += a * x with a = a.hi + a.lo, x = x.hi + x.lo (drops lo*lo).
SKL_DEV void ff_fma(ff& acc, ff a, ff x)
{
    float p = __fmul_rn(a.hi, x.hi);
    float pe = __fmaf_rn(a.hi, x.hi, -p);
    float pl = __fmaf_rn(a.hi, x.lo, __fmaf_rn(a.lo, x.hi, pe));
    ff_add(acc, p, pl);
}

SKL_DEV ff ff_shfl_xor(ff a, int lane_mask)
{
    return {__shfl_xor_sync(0xffffffffu, a.hi, lane_mask), __shfl_xor_sync(0xffffffffu, a.lo, lane_mask)};
}

SKL_DEV ff warp_sum_ff(ff a)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ff_add(a, ff_shfl_xor(a, o));
    return a;
}

// ------------------------------------------------------------ reductions --
template <typename T>
SKL_DEV T warp_sum(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <typename T>
SKL_DEV T warp_max(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        T w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

// Block-wide sum; scratch must hold blockDim.x/32 values.  All threads get it.
template <typename T>
SKL_DEV T block_sum(T v, T* scratch)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) scratch[wid] = v;
    __syncthreads();
    T t = (threadIdx.x < nw) ? scratch[threadIdx.x] : T(0);
    if (wid == 0) t = warp_sum(t);
    if (threadIdx.x == 0) scratch[0] = t;
    __syncthreads();
    T r = scratch[0];
    __syncthreads();
    return r;
}

template <typename T>
SKL_DEV T block_max(T v, T* scratch)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_max(v);
    __syncthreads();
    if (lane == 0) scratch[wid] = v;
    __syncthreads();
    T t = (threadIdx.x < nw) ? scratch[threadIdx.x] : T(0);
    if (wid == 0) t = warp_max(t);
    if (threadIdx.x == 0) scratch[0] = t;
    __syncthreads();
    T r = scratch[0];
    __syncthreads();
    return r;
}

SKL_DEV ff block_sum_ff(ff v, ff* scratch)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_sum_ff(v);
    __syncthreads();
    if (lane == 0) scratch[wid] = v;
    __syncthreads();
    ff t = (threadIdx.x < nw) ? scratch[threadIdx.x] : ff{0.f, 0.f};
    if (wid == 0) t = warp_sum_ff(t);
    if (threadIdx.x == 0) scratch[0] = t;
    __syncthreads();
    ff r = scratch[0];
    __syncthreads();
    return r;
}

// ---------------------------------------------------------- device status --
// Device-side error word: kernels OR in a code, the host reads it at its next
// synchronisation point.  Waits never spin without a bound.
enum : unsigned {
    kDevErrTimeout = 1u,
    kDevErrBounds = 2u,
    kDevErrNumeric = 4u,
    kDevErrQrSelect = 8u,   // the sample QRP picked an invalid column (non-finite sketch)
};

constexpr long long kSpinLimit = 1ll << 24;

SKL_DEV void dev_flag(unsigned* status, unsigned code)
{
    if (status) atomicOr(status, code);
}

// ---------------------------------------------------------- cluster (DSMEM) --
SKL_DEV unsigned cluster_ctarank()
{
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

SKL_DEV unsigned cluster_nctarank()
{
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}

SKL_DEV void cluster_sync()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\t"
                 "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Map a local shared-memory address to the same offset in CTA `rank` of the
// cluster and load a float / int / double from it.
SKL_DEV uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

SKL_DEV uint32_t dsmem_addr(const void* local, unsigned rank)
{
    uint32_t a = smem_u32(local), r;
    asm("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
    return r;
}

// The loads are volatile (never merged, hoisted or dropped, and kept in order
// relative to the cluster barriers, which carry the memory clobber) but carry
// no clobber themselves, so independent loads issue back to back and their
// latencies overlap.
SKL_DEV float dsmem_ld_f32(const float* local, unsigned rank)
{
    float v;
    asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(dsmem_addr(local, rank)));
    return v;
}

SKL_DEV double dsmem_ld_f64(const double* local, unsigned rank)
{
    double v;
    asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(dsmem_addr(local, rank)));
    return v;
}

SKL_DEV int dsmem_ld_s32(const int* local, unsigned rank)
{
    int v;
    asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(dsmem_addr(local, rank)));
    return v;
}

// Remote stores (fire and forget; a later cluster barrier with release /
// acquire semantics orders them for the destination CTA).
SKL_DEV void dsmem_st_f32(float* local, unsigned rank, float v)
{
    asm volatile("st.shared::cluster.f32 [%0], %1;" :: "r"(dsmem_addr(local, rank)), "f"(v) : "memory");
}
SKL_DEV void dsmem_st_f64(double* local, unsigned rank, double v)
{
    asm volatile("st.shared::cluster.f64 [%0], %1;" :: "r"(dsmem_addr(local, rank)), "d"(v) : "memory");
}
SKL_DEV void dsmem_st_s32(int* local, unsigned rank, int v)
{
    asm volatile("st.shared::cluster.s32 [%0], %1;" :: "r"(dsmem_addr(local, rank)), "r"(v) : "memory");
}
// 16-byte remote store; `local` must be 16-byte aligned.
SKL_DEV void dsmem_st_v4f32(float* local, unsigned rank, float4 v)
{
    asm volatile("st.shared::cluster.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(dsmem_addr(local, rank)),
                 "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w)
                 : "memory");
}
SKL_DEV void dsmem_st(float* local, unsigned rank, float v) { dsmem_st_f32(local, rank, v); }
SKL_DEV void dsmem_st(double* local, unsigned rank, double v) { dsmem_st_f64(local, rank, v); }

template <typename T>
SKL_DEV T dsmem_ld(const T* local, unsigned rank);
template <>
SKL_DEV float dsmem_ld<float>(const float* local, unsigned rank) { return dsmem_ld_f32(local, rank); }
template <>
SKL_DEV double dsmem_ld<double>(const double* local, unsigned rank) { return dsmem_ld_f64(local, rank); }

// Scalar helpers usable for float and double.
template <typename T> SKL_DEV T t_abs(T x) { return x < T(0) ? -x : x; }
template <typename T> SKL_DEV T t_sqrt(T x);
template <> SKL_DEV float t_sqrt<float>(float x) { return sqrtf(x); }
template <> SKL_DEV double t_sqrt<double>(double x) { return sqrt(x); }

}  // namespace skl
