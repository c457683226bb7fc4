// k_sketch.cu -- s-hashing sketch S*A, S*b (sparse path).
//
// Reference: sparse_sketch (src/sketching.cpp:90-112) builds S with
// gen_hashing_matrix and forms S*A with CSparse's cs_dl_multiply and S*b with
// cs_dl_gaxpy.  Here one CTA owns one column j of A: its nonzeros are read
// once from HBM (int32 row index + FP64 value, 12 B/nnz) and scattered into
// a shared-memory column of length m.  The accumulation is done in 64-bit
// fixed point scaled to the column's largest magnitude, so collisions sum
// exactly and the result does not depend on the order of the atomics; the
// column is then written once, coalesced, already multiplied by 1/sqrt(k)
// and (optionally) by 1/||A(:,j)||_2 (column equilibration, folded back into
// the preconditioner).  S*b is a fixed-order gather over the bucket lists of
// S, in the same order and arithmetic as cs_dl_gaxpy.
#include <cmath>

#include "skl_internal.hpp"
#include "launch.cuh"
#include "common.cuh"

namespace skl {

constexpr int kSketchThreads = 512;

template <typename T, int NT>
__global__ void __launch_bounds__(NT)
k_sketch_sparse_smem(const int* __restrict__ cp, const int* __restrict__ ri,
                     const double* __restrict__ Ax, const unsigned* __restrict__ hidx, int k,
                     int m, T* __restrict__ SA, int64_t ld, int equilibrate, double inv_sqrt_k,
                     double* __restrict__ colnorm, double* __restrict__ colscale)
{
    pdl_wait();
    extern __shared__ unsigned long long acc[];   // m entries
    __shared__ double s_red[NT / 32];
    const int j = blockIdx.x;
    const int p0 = cp[j], p1 = cp[j + 1];
    for (int h = threadIdx.x; h < m; h += blockDim.x) acc[h] = 0ull;

    double mx = 0.0, ss = 0.0;
    for (int p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
        double a = Ax[p];
        double aa = fabs(a);
        mx = aa > mx ? aa : mx;
        ss = fma(a, a, ss);
    }
    mx = block_max(mx, s_red);
    ss = block_sum(ss, s_red);
    const int cnt = p1 - p0;
    // 2^sh * max|a| < 2^(62 - ceil(log2(cnt*k))) keeps every partial sum in range.
    int emax = 0;
    frexp(mx, &emax);
    int guard = 1;
    while ((1ll << guard) < (long long)cnt * k + 1) ++guard;
    const int sh = 62 - guard - emax;
    for (int p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
        long long q = llrint(ldexp(Ax[p], sh));
        const unsigned* hp = hidx + (int64_t)ri[p] * k;
        for (int t = 0; t < k; ++t) {
            unsigned e = hp[t];
            long long v = (e & 0x80000000u) ? -q : q;
            atomicAdd(&acc[e & 0x7fffffffu], (unsigned long long)v);
        }
    }
    __syncthreads();
    double nrm = sqrt(ss);
    double cs = (equilibrate && nrm > 0.0) ? 1.0 / nrm : 1.0;
    if (threadIdx.x == 0) {
        colnorm[j] = nrm;
        colscale[j] = cs;
    }
    const double f = ldexp(inv_sqrt_k * cs, -sh);
    T* out = SA + (int64_t)j * ld;
    for (int h = threadIdx.x; h < m; h += blockDim.x)
        out[h] = (T)((double)(long long)acc[h] * f);
}

// Large m (shared column does not fit): accumulate in a global FP64 column
// buffer with the same fixed-point rule, one CTA per column, columns processed
// in slices so the global scratch stays bounded.
template <typename T>
__global__ void __launch_bounds__(kSketchThreads)
k_sketch_sparse_global(const int* __restrict__ cp, const int* __restrict__ ri,
                       const double* __restrict__ Ax, const unsigned* __restrict__ hidx, int k,
                       int m, T* __restrict__ SA, int64_t ld, int equilibrate, double inv_sqrt_k,
                       double* __restrict__ colnorm, double* __restrict__ colscale,
                       unsigned long long* __restrict__ scratch, int col0)
{
    pdl_wait();
    __shared__ double s_red[kSketchThreads / 32];
    const int j = col0 + blockIdx.x;
    unsigned long long* acc = scratch + (int64_t)blockIdx.x * m;
    const int p0 = cp[j], p1 = cp[j + 1];
    for (int h = threadIdx.x; h < m; h += blockDim.x) acc[h] = 0ull;
    double mx = 0.0, ss = 0.0;
    for (int p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
        double a = Ax[p];
        mx = fabs(a) > mx ? fabs(a) : mx;
        ss = fma(a, a, ss);
    }
    mx = block_max(mx, s_red);
    ss = block_sum(ss, s_red);
    const int cnt = p1 - p0;
    int emax = 0;
    frexp(mx, &emax);
    int guard = 1;
    while ((1ll << guard) < (long long)cnt * k + 1) ++guard;
    const int sh = 62 - guard - emax;
    __syncthreads();
    for (int p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
        long long q = llrint(ldexp(Ax[p], sh));
        const unsigned* hp = hidx + (int64_t)ri[p] * k;
        for (int t = 0; t < k; ++t) {
            unsigned e = hp[t];
            long long v = (e & 0x80000000u) ? -q : q;
            atomicAdd(&acc[e & 0x7fffffffu], (unsigned long long)v);
        }
    }
    __syncthreads();
    double nrm = sqrt(ss);
    double cs = (equilibrate && nrm > 0.0) ? 1.0 / nrm : 1.0;
    if (threadIdx.x == 0) {
        colnorm[j] = nrm;
        colscale[j] = cs;
    }
    const double f = ldexp(inv_sqrt_k * cs, -sh);
    T* out = SA + (int64_t)j * ld;
    for (int h = threadIdx.x; h < m; h += blockDim.x)
        out[h] = (T)((double)(long long)acc[h] * f);
}

// Opt-in shared memory per block (the same on every GB300), read once; the
// initialisation is thread-safe for concurrent solves.
static size_t smem_optin()
{
    static const size_t v = [] {
        int dev = 0, o = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&o, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        return (size_t)o;
    }();
    return v;
}

template <typename T, int NT>
static void launch_sketch_smem(const int* cp, const int* ri, const double* Ax, int64_t d,
                               const unsigned* hidx, int k, int64_t m, T* SA, int64_t ld,
                               int equilibrate, double isk, double* colnorm, double* colscale,
                               size_t smem, cudaStream_t st)
{
    allow_max_dynamic_smem((const void*)k_sketch_sparse_smem<T, NT>);
    launch_k(k_sketch_sparse_smem<T, NT>, (unsigned)d, NT, smem, st, cp, ri, Ax, hidx, k, (int)m, SA, ld,
                                                               equilibrate, isk, colnorm, colscale);
    SKL_LAUNCHED();
}

template <typename T>
void sketch_sparse(const int* cp, const int* ri, const double* Ax, int64_t n, int64_t d,
                   const unsigned* hidx, int k, int64_t m, T* SA, int64_t ld, int equilibrate,
                   double* colnorm, double* colscale, cudaStream_t st, int threads)
{
    (void)n;
    if (d <= 0) return;
    const double isk = 1.0 / std::sqrt((double)k);
    size_t smem = (size_t)m * sizeof(unsigned long long);
    if (smem + 1024 <= smem_optin()) {
        // one CTA per column of A; the block size is a tuning choice (S A is
        // accumulated exactly in fixed point; only the order in which the
        // column norm's squares are summed depends on it)
        if (threads == 256)
            launch_sketch_smem<T, 256>(cp, ri, Ax, d, hidx, k, m, SA, ld, equilibrate, isk, colnorm,
                                       colscale, smem, st);
        else if (threads == 1024)
            launch_sketch_smem<T, 1024>(cp, ri, Ax, d, hidx, k, m, SA, ld, equilibrate, isk, colnorm,
                                        colscale, smem, st);
        else
            launch_sketch_smem<T, kSketchThreads>(cp, ri, Ax, d, hidx, k, m, SA, ld, equilibrate, isk,
                                                  colnorm, colscale, smem, st);
        return;
    }
    // Bounded global scratch: up to 256 columns in flight per launch.
    const int slice = 256;
    unsigned long long* scratch = nullptr;
    SKL_CUDA(cudaMallocAsync(&scratch, (size_t)slice * m * sizeof(unsigned long long), st));
    for (int64_t c0 = 0; c0 < d; c0 += slice) {
        int nc = (int)((d - c0) < slice ? (d - c0) : slice);
        launch_k(k_sketch_sparse_global<T>, nc, kSketchThreads, 0, st, 
            cp, ri, Ax, hidx, k, (int)m, SA, ld, equilibrate, isk, colnorm, colscale, scratch,
            (int)c0);
        SKL_LAUNCHED();
    }
    SKL_CUDA(cudaFreeAsync(scratch, st));
}

template void sketch_sparse<float>(const int*, const int*, const double*, int64_t, int64_t,
                                   const unsigned*, int, int64_t, float*, int64_t, int, double*,
                                   double*, cudaStream_t, int);
template void sketch_sparse<double>(const int*, const int*, const double*, int64_t, int64_t,
                                    const unsigned*, int, int64_t, double*, int64_t, int, double*,
                                    double*, cudaStream_t, int);

// S*b: Sb[h] = sum over the bucket of h, in increasing source row, of
// (+-1/sqrt(k)) * b[i] -- the order and arithmetic of cs_dl_gaxpy.
__global__ void k_sketch_rhs(const int* __restrict__ bptr, const unsigned* __restrict__ bent,
                             int m, double v, const double* __restrict__ b,
                             double* __restrict__ Sb)
{
    pdl_wait();
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < m; h += gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int q = bptr[h]; q < bptr[h + 1]; ++q) {
            unsigned e = bent[q];
            double s = (e & 0x80000000u) ? -v : v;
            acc = __dadd_rn(acc, __dmul_rn(s, b[e & 0x7fffffffu]));
        }
        Sb[h] = acc;
    }
}

void sketch_rhs(const int* bptr, const unsigned* bent, int64_t m, int k, const double* b,
                double* Sb, cudaStream_t st)
{
    const double v = 1.0 / std::sqrt((double)k);
    unsigned g = (unsigned)((m + 255) / 256);
    launch_k(k_sketch_rhs, g, 256, 0, st, bptr, bent, (int)m, v, b, Sb);
    SKL_LAUNCHED();
}

}  // namespace skl
