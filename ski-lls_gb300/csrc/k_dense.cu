// k_dense.cu -- randomized Hartley transform + hashing sketch for dense A.
//
// Reference: rand_hashing_dct (src/dense_helpers.cpp:83-112):
//   D = random signs (gen_scaled_rand_signs, :7-16),
//   Y = DHT_N( D * A / sqrt(N) ) column by column (fast_unitary_transform,
//       src/fast_unitary_transform.cpp:42-121, FFTW_DHT via fftw_r2r.cpp:33-51),
//   SA = (1/sqrt(k)) * S * Y  with S's values +-1/sqrt(k)  (sketch(),
//       src/sketching.cpp:39-62), same for b.
//
// GB300 mapping: one CTA per column.  The column is read once from HBM
// (multiplied by D/sqrt(N) on load), transformed in shared memory, and hashed
// into its m sketch rows by a fixed-order gather over S's bucket lists, so
// HDA never exists in HBM.  The DHT of a real length-N vector is computed from
// a complex FFT of half length L = N/2 (even/odd packing) and H = Re F - Im F.
// The FFT is a Stockham autosort pass sequence with radices 7, 5, 4, 3, 2:
// FP32 columns stay in shared memory (each pass reads its butterflies into
// registers, synchronises, writes back in place); FP64 columns, or lengths
// beyond shared memory, ping-pong through a global scratch slab per CTA.
#include <cmath>

#include "skl_internal.hpp"
#include "launch.cuh"
#include "common.cuh"

namespace skl {

constexpr int kFftThreads = 1024;
constexpr int kFftMaxPerThread = 32;            // complex values per thread (registers)
constexpr int kFftMaxRadices = 32;
constexpr int kFftDhtStage = 26;               // unpack values per thread (L <= 26 * 1024)
constexpr int kFftSmemMaxL = 25 * 1024;        // shared-memory path limit

template <typename T> struct Cplx;
template <> struct Cplx<float> { using type = float2; };
template <> struct Cplx<double> { using type = double2; };

template <typename C> SKL_DEV C cmk(double re, double im);
template <> SKL_DEV float2 cmk<float2>(double re, double im) { return make_float2((float)re, (float)im); }
template <> SKL_DEV double2 cmk<double2>(double re, double im) { return make_double2(re, im); }
template <typename C> SKL_DEV C cadd(C a, C b) { a.x += b.x; a.y += b.y; return a; }
template <typename C> SKL_DEV C csub(C a, C b) { a.x -= b.x; a.y -= b.y; return a; }
template <typename C> SKL_DEV C cmul(C a, C b)
{
    C r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}

// exp(-2 pi i * num / den) in the working precision, 0 <= num < den < 2^31
// (32-bit operands: a 64-bit remainder or division per twiddle is a long
// emulated sequence).
template <typename T>
SKL_DEV typename Cplx<T>::type twiddle(int num, int den)
{
    if constexpr (std::is_same<T, float>::value) {
        float s, c;
        sincospif(-2.0f * (float)num / (float)den, &s, &c);
        return make_float2(c, s);
    } else {
        double s, c;
        sincospi(-2.0 * (double)num / (double)den, &s, &c);
        return make_double2(c, s);
    }
}

// The R-th roots of unity of the small DFTs, exp(-2 pi i j / R), as compile-
// time constants: cos and sin by their Taylor series (the argument reduced to
// [-pi, pi], 30 terms: far below double rounding there), so the radix-3/5/7
// butterflies carry no runtime trigonometry.
constexpr double kPiD = 3.14159265358979323846;
constexpr double cx_sin(double x)
{
    double term = x, sum = x;
    for (int n = 1; n < 30; ++n) {
        term *= -x * x / ((2.0 * n) * (2.0 * n + 1.0));
        sum += term;
    }
    return sum;
}
constexpr double cx_cos(double x)
{
    double term = 1.0, sum = 1.0;
    for (int n = 1; n < 30; ++n) {
        term *= -x * x / ((2.0 * n - 1.0) * (2.0 * n));
        sum += term;
    }
    return sum;
}
constexpr double root_angle(int j, int R)
{
    const double a = -2.0 * kPiD * (double)(j % R) / (double)R;
    return a < -kPiD ? a + 2.0 * kPiD : a;
}
template <int R>
struct Roots {
    double re[R], im[R];
    constexpr Roots() : re(), im()
    {
        for (int j = 0; j < R; ++j) {
            re[j] = cx_cos(root_angle(j, R));
            im[j] = cx_sin(root_angle(j, R));
        }
    }
};
template <typename T, int R>
SKL_DEV typename Cplx<T>::type small_root(int j)
{
    constexpr Roots<R> w{};
    typename Cplx<T>::type r;
    r.x = (T)w.re[j % R];
    r.y = (T)w.im[j % R];
    return r;
}

// In-register R-point DFT (forward) of v[0..R).
template <typename T, int R>
SKL_DEV void dft_small(typename Cplx<T>::type* v)
{
    using C = typename Cplx<T>::type;
    if constexpr (R == 2) {
        C a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    } else if constexpr (R == 4) {
        C a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
        C b0 = cadd(v[1], v[3]), b1 = csub(v[1], v[3]);
        // -i * b1
        C mb1;
        mb1.x = b1.y;
        mb1.y = -b1.x;
        v[0] = cadd(a0, b0);
        v[2] = csub(a0, b0);
        v[1] = cadd(a1, mb1);
        v[3] = csub(a1, mb1);
    } else {
        C out[R];
#pragma unroll
        for (int q = 0; q < R; ++q) {
            C acc = v[0];
#pragma unroll
            for (int t = 1; t < R; ++t) acc = cadd(acc, cmul(v[t], small_root<T, R>(q * t)));
            out[q] = acc;
        }
#pragma unroll
        for (int q = 0; q < R; ++q) v[q] = out[q];
    }
}

// Butterfly i of a radix-R Stockham pass with parameter p (product of the
// radices already applied): inputs x[i + q*L/R], twiddles exp(-2 pi i q k/(pR)),
// outputs y[(i-k)*R + k + q*p], k = i mod p.
template <typename T, int R>
SKL_DEV void butterfly_load(const typename Cplx<T>::type* x, int L, int p, int i,
                            typename Cplx<T>::type* v)
{
    const int T_ = L / R;
    const int k = i % p;
#pragma unroll
    for (int q = 0; q < R; ++q) v[q] = x[i + q * T_];
    if (p > 1 && k > 0) {
        // w^q for w = exp(-2 pi i k / (pR)): one sincospi, then powers
        const typename Cplx<T>::type w = twiddle<T>(k, p * R);
        typename Cplx<T>::type wq = w;
#pragma unroll
        for (int q = 1; q < R; ++q) {
            v[q] = cmul(v[q], wq);
            if (q + 1 < R) wq = cmul(wq, w);
        }
    }
    dft_small<T, R>(v);
}

template <typename T, int R>
SKL_DEV void butterfly_store(typename Cplx<T>::type* y, int p, int i, const typename Cplx<T>::type* v)
{
    const int k = i % p;
    const int j = (i - k) * R + k;
#pragma unroll
    for (int q = 0; q < R; ++q) y[j + q * p] = v[q];
}

// One pass in place on `buf` (all threads load, sync, store).
template <typename T, int R>
SKL_DEV void pass_inplace(typename Cplx<T>::type* buf, int L, int p)
{
    using C = typename Cplx<T>::type;
    const int nb = L / R;
    C v[kFftMaxPerThread];
    int cnt = 0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        butterfly_load<T, R>(buf, L, p, i, v + cnt * R);
        ++cnt;
    }
    __syncthreads();
    cnt = 0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        butterfly_store<T, R>(buf, p, i, v + cnt * R);
        ++cnt;
    }
    __syncthreads();
}

template <typename T, int R>
SKL_DEV void pass_pingpong(const typename Cplx<T>::type* x, typename Cplx<T>::type* y, int L, int p)
{
    using C = typename Cplx<T>::type;
    const int nb = L / R;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {
        C v[R];
        butterfly_load<T, R>(x, L, p, i, v);
        butterfly_store<T, R>(y, p, i, v);
    }
    __syncthreads();
}

struct FftPlan {
    int L;
    int nr;
    int radix[kFftMaxRadices];
};

// Complex forward FFT of length L on buf (in place for shared memory; with a
// second buffer `alt` the passes ping-pong and the result ends in *res).
template <typename T>
SKL_DEV typename Cplx<T>::type* fft_run(const FftPlan& P, typename Cplx<T>::type* buf,
                                        typename Cplx<T>::type* alt)
{
    using C = typename Cplx<T>::type;
    int p = 1;
    C* x = buf;
    C* y = alt;
    for (int s = 0; s < P.nr; ++s) {
        const int R = P.radix[s];
        if (!alt) {
            switch (R) {
            case 2: pass_inplace<T, 2>(x, P.L, p); break;
            case 3: pass_inplace<T, 3>(x, P.L, p); break;
            case 4: pass_inplace<T, 4>(x, P.L, p); break;
            case 5: pass_inplace<T, 5>(x, P.L, p); break;
            default: pass_inplace<T, 7>(x, P.L, p); break;
            }
        } else {
            switch (R) {
            case 2: pass_pingpong<T, 2>(x, y, P.L, p); break;
            case 3: pass_pingpong<T, 3>(x, y, P.L, p); break;
            case 4: pass_pingpong<T, 4>(x, y, P.L, p); break;
            case 5: pass_pingpong<T, 5>(x, y, P.L, p); break;
            default: pass_pingpong<T, 7>(x, y, P.L, p); break;
            }
            C* t = x;
            x = y;
            y = t;
        }
        p *= R;
    }
    return x;
}

// Column transform.  Input column a (n entries, FP64) times D/sqrt(N), zero
// padded to N = 2L; output H (N reals) written over the complex buffer as
// reals (H[k] at ((T*)buf)[k]) -- the caller provides the buffers.
template <typename T>
SKL_DEV typename Cplx<T>::type* dht_column(const FftPlan& P, const double* __restrict__ a, int n,
                                           const double* __restrict__ D, double scale,
                                           typename Cplx<T>::type* buf,
                                           typename Cplx<T>::type* alt)
{
    using C = typename Cplx<T>::type;
    const int L = P.L;
    // pack z[t] = x[2t] + i x[2t+1]
    const T sc = (T)scale;
    for (int t = threadIdx.x; t < L; t += blockDim.x) {
        const int i0 = 2 * t, i1 = 2 * t + 1;
        T x0 = i0 < n ? (T)a[i0] : T(0);
        T x1 = i1 < n ? (T)a[i1] : T(0);
        if (i0 < n && D[i0] < 0) x0 = -x0;
        if (i1 < n && D[i1] < 0) x1 = -x1;
        C z;
        z.x = x0 * sc;
        z.y = x1 * sc;
        buf[t] = z;
    }
    __syncthreads();
    C* Z = fft_run<T>(P, buf, alt);
    // unpack: X[k] = (Z[k] + conj(Z[L-k]))/2 - i/2 e^{-2 pi i k/N} (Z[k] - conj(Z[L-k]))
    // H[k] = Re X[k] - Im X[k] (k < L), H[N-k] = Re X[k] + Im X[k] (0 < k < L),
    // H[L] = Re Z[0] - Im Z[0].
    const int N = 2 * L;
    auto hvals = [&](int kk, T& hk, T& hnk) {
        const C zk = Z[kk % L];
        const C zc = Z[(L - kk) % L];
        const T er = (zk.x + zc.x) * T(0.5), ei = (zk.y - zc.y) * T(0.5);   // even part
        const T or_ = (zk.y + zc.y) * T(0.5), oi = -(zk.x - zc.x) * T(0.5); // odd part
        const C w = twiddle<T>(kk, 2 * L);
        const T xr = er + (w.x * or_ - w.y * oi);
        const T xi = ei + (w.x * oi + w.y * or_);
        hk = xr - xi;
        hnk = xr + xi;
    };
    if (alt) {
        // ping-pong path: write the reals into the other buffer
        C* other = (Z == buf) ? alt : buf;
        T* H = reinterpret_cast<T*>(other);
        for (int kk = threadIdx.x; kk < L; kk += blockDim.x) {
            T hk, hnk;
            hvals(kk, hk, hnk);
            H[kk] = hk;
            if (kk != 0) H[N - kk] = hnk;
        }
        if (threadIdx.x == 0) H[L] = Z[0].x - Z[0].y;
        __syncthreads();
        return other;
    }
    // in place (shared memory): stage in registers, synchronise, write
    T hv[2 * kFftDhtStage];
    int cnt = 0;
    for (int kk = threadIdx.x; kk < L; kk += blockDim.x) {
        hvals(kk, hv[cnt], hv[cnt + 1]);
        cnt += 2;
    }
    T hL = T(0);
    if (threadIdx.x == 0) hL = Z[0].x - Z[0].y;
    __syncthreads();
    T* H = reinterpret_cast<T*>(Z);
    cnt = 0;
    for (int kk = threadIdx.x; kk < L; kk += blockDim.x) {
        H[kk] = hv[cnt];
        if (kk != 0) H[N - kk] = hv[cnt + 1];
        cnt += 2;
    }
    if (threadIdx.x == 0) H[L] = hL;
    __syncthreads();
    return Z;
}

template <typename T>
__global__ void __launch_bounds__(kFftThreads)
k_dht_hash(const double* __restrict__ A, int64_t lda, int n, int d, const double* __restrict__ D,
           FftPlan P, double scale, const int* __restrict__ bptr, const unsigned* __restrict__ bent,
           int m, double alpha_v, T* __restrict__ SA, int64_t ld, double* __restrict__ Yout,
           int64_t ldy, typename Cplx<T>::type* __restrict__ gscratch)
{
    pdl_wait();
    using C = typename Cplx<T>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* buf;
    C* alt = nullptr;
    if (gscratch) {
        buf = gscratch + (size_t)blockIdx.x * 2 * P.L;
        alt = buf + P.L;
    } else {
        buf = reinterpret_cast<C*>(smem_raw);
    }
    const int N = 2 * P.L;
    for (int j = blockIdx.x; j < d; j += gridDim.x) {
        C* Z = dht_column<T>(P, A + (int64_t)j * lda, n, D, scale, buf, alt);
        const T* H = reinterpret_cast<const T*>(Z);
        if (Yout) {
            for (int k = threadIdx.x; k < N; k += blockDim.x) Yout[k + (int64_t)j * ldy] = (double)H[k];
        }
        if (SA) {
            // SA[h, j] = sum over the bucket of h (increasing source row) of
            // alpha * (+-1/sqrt(k)) * H[i]  -- the order of csc_mv 'n'
            const T av = (T)alpha_v;
            for (int h = threadIdx.x; h < m; h += blockDim.x) {
                T acc = T(0);
                for (int q = bptr[h]; q < bptr[h + 1]; ++q) {
                    const unsigned e = bent[q];
                    const T hv = H[e & 0x7fffffffu];
                    acc += (e & 0x80000000u) ? -av * hv : av * hv;
                }
                SA[h + (int64_t)j * ld] = acc;
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------ host side --
static bool factor_plan(int64_t L, FftPlan& P)
{
    P.L = (int)L;
    P.nr = 0;
    int64_t r = L;
    const int pref[] = {4, 2, 3, 5, 7};
    for (int f : {7, 5, 3}) {
        while (r % f == 0) {
            if (P.nr >= kFftMaxRadices) return false;
            P.radix[P.nr++] = f;
            r /= f;
        }
    }
    while (r % 4 == 0) {
        if (P.nr >= kFftMaxRadices) return false;
        P.radix[P.nr++] = 4;
        r /= 4;
    }
    while (r % 2 == 0) {
        if (P.nr >= kFftMaxRadices) return false;
        P.radix[P.nr++] = 2;
        r /= 2;
    }
    (void)pref;
    return r == 1;
}

static bool smooth(int64_t x)
{
    for (int f : {2, 3, 5, 7})
        while (x % f == 0) x /= f;
    return x == 1;
}

// Transform length: N = n when n is even and n/2 factors into 2,3,5,7;
// otherwise (or with wisdom) the next such even length >= n.  Zero padding
// keeps the transform orthonormal (the reference pads in its wisdom mode,
// src/fast_unitary_transform.cpp:63-64,98-99).
int64_t dht_length(int64_t n, int wisdom)
{
    int64_t N = n + (n & 1);
    if (!wisdom && smooth(N / 2)) return N;
    while (!smooth(N / 2)) N += 2;
    return N;
}

// Opt-in shared memory per block (the same on every GB300), read once; the
// initialisation is thread-safe for concurrent solves.
static size_t smem_optin_bytes()
{
    static const size_t v = [] {
        int dev = 0, o = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&o, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        return (size_t)o;
    }();
    return v;
}

template <typename T>
static void launch_dht(const double* A, int64_t lda, int64_t n, int64_t d, const double* D,
                       int64_t N, const int* bptr, const unsigned* bent, int k, int64_t m, T* SA,
                       int64_t ld, double* Yout, int64_t ldy, void* gscratch_buf,
                       size_t gscratch_bytes, cudaStream_t st)
{
    using C = typename Cplx<T>::type;
    FftPlan P;
    if (N & 1) fail(SKL_ERR_INVALID, "DHT length must be even");
    if (!factor_plan(N / 2, P)) fail(SKL_ERR_INVALID, "DHT length must factor into 2,3,5,7");
    const size_t need = (size_t)P.L * sizeof(C);
    const bool in_smem = std::is_same<T, float>::value && need + 1024 <= smem_optin_bytes() &&
                         P.L <= kFftSmemMaxL;
    const double scale = 1.0 / std::sqrt((double)N);
    const double alpha_v = (1.0 / std::sqrt((double)k)) * (1.0 / std::sqrt((double)k));
    unsigned grid = (unsigned)std::min<int64_t>(d, 152);
    if (in_smem) {
        allow_max_dynamic_smem((const void*)k_dht_hash<T>);
        launch_k(k_dht_hash<T>, grid, kFftThreads, need, st, A, lda, (int)n, (int)d, D, P, scale, bptr,
                                                        bent, (int)m, alpha_v, SA, ld, Yout, ldy,
                                                        nullptr);
    } else {
        const size_t per = 2 * (size_t)P.L * sizeof(C);
        grid = (unsigned)std::min<int64_t>(grid, (int64_t)(gscratch_bytes / per));
        if (grid == 0) fail(SKL_ERR_ALLOC, "DHT scratch too small");
        launch_k(k_dht_hash<T>, grid, kFftThreads, 0, st, A, lda, (int)n, (int)d, D, P, scale, bptr, bent,
                                                     (int)m, alpha_v, SA, ld, Yout, ldy,
                                                     (C*)gscratch_buf);
    }
    SKL_LAUNCHED();
}

void dht_load_kernels()
{
    cudaFuncAttributes fa;
    SKL_CUDA(cudaFuncGetAttributes(&fa, k_dht_hash<float>));
    SKL_CUDA(cudaFuncGetAttributes(&fa, k_dht_hash<double>));
}

size_t dht_scratch_bytes(int64_t N, int precision)
{
    const size_t csz = precision == SKL_PREC_FP64 ? sizeof(double2) : sizeof(float2);
    return (size_t)152 * 2 * (size_t)(N / 2) * csz;
}

template <typename T>
void dht_hash(const double* A, int64_t lda, int64_t n, int64_t d, const double* D, int64_t N,
              const int* bptr, const unsigned* bent, int k, int64_t m, T* SA, int64_t ld,
              double* Yout, int64_t ldy, void* scratch, size_t scratch_bytes, cudaStream_t st)
{
    launch_dht<T>(A, lda, n, d, D, N, bptr, bent, k, m, SA, ld, Yout, ldy, scratch, scratch_bytes, st);
}

template void dht_hash<float>(const double*, int64_t, int64_t, int64_t, const double*, int64_t,
                              const int*, const unsigned*, int, int64_t, float*, int64_t, double*,
                              int64_t, void*, size_t, cudaStream_t);
template void dht_hash<double>(const double*, int64_t, int64_t, int64_t, const double*, int64_t,
                               const int*, const unsigned*, int, int64_t, double*, int64_t,
                               double*, int64_t, void*, size_t, cudaStream_t);

// Sb: the same transform of b (one column, FP64 arithmetic) and bucket gather.
void dht_hash_rhs(const double* b, int64_t n, const double* D, int64_t N, const int* bptr,
                  const unsigned* bent, int k, int64_t m, double* Sb, void* scratch,
                  size_t scratch_bytes, cudaStream_t st)
{
    launch_dht<double>(b, n, n, 1, D, N, bptr, bent, k, m, Sb, m, nullptr, 0, scratch,
                       scratch_bytes, st);
}

// Per-block partial sums of squares of a dense column-major matrix (512
// blocks): FP32 sums per thread, FP64 per block -- ||A||_F only normalises the
// reported backward error.
__global__ void k_fro_partial(const double* __restrict__ A, int64_t lda, int64_t n, int64_t d,
                              double* __restrict__ out)
{
    pdl_wait();
    __shared__ double red[32];
    double acc = 0.0;
    for (int64_t j = blockIdx.x; j < d; j += gridDim.x) {
        float s = 0.f;
        for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
            float v = (float)A[i + j * lda];
            s = fmaf(v, v, s);
        }
        acc += (double)s;
    }
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) out[blockIdx.x] = acc;
}

void fro_partials(const double* A, int64_t lda, int64_t n, int64_t d, double* out512,
                  cudaStream_t st)
{
    SKL_CUDA(cudaMemsetAsync(out512, 0, 512 * sizeof(double), st));
    launch_k(k_fro_partial, 512, 256, 0, st, A, lda, n, d, out512);
    SKL_LAUNCHED();
}

}  // namespace skl
