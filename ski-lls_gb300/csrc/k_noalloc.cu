// k_noalloc.cu -- skl_dht_device_noalloc: the column DHT of the dense path on
// caller-owned device buffers, with its FFT ping-pong scratch taken from a
// fixed static device array instead of the library's arena.  It calls no
// cudaMalloc/cudaFree and no other allocating routine.
//
// Who needs it: callers that cannot let a library allocate device memory --
// a host framework whose caching allocator already owns (nearly) all of the
// device, code that must keep a fixed device footprint known when the library
// is loaded, and latency-critical loops where a cudaFree (which synchronises
// the whole device) would stall every other stream.
//
// The scratch array lives in this translation unit alone, so with CUDA's lazy
// module loading (the default) its memory is committed on a device only once
// this entry point is used there; with CUDA_MODULE_LOADING=EAGER every device
// the process initialises commits it when the library's module loads.
// The device address is looked up once per device and kept; after
// cudaDeviceReset call skl_finalize() (which forgets it) before using this
// entry point again.
#include <cstdint>
#include <mutex>
#include <string>

#include "skl_internal.hpp"

namespace skl {

// 64 MiB: the ping-pong pair of one column is 2 * (N/2) complex values
// (16 N bytes in FP64, 8 N in FP32), so N <= 4,194,304 fits one column and
// the number of columns transformed at once is min(d, 152, 64 MiB / that).
constexpr size_t kDhtNoallocScratchBytes = (size_t)SKL_DHT_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

// Nothing in it needs to start at zero: each column's buffers are written in
// full (the zero-padded input pack, every FFT pass, the real unpack) before
// they are read.
static __device__ __align__(256) unsigned char g_dht_scratch[kDhtNoallocScratchBytes];

static std::mutex g_setup_mu;
static void* g_scratch_ptr[kMaxDevices];

// One-time set-up on the current device: resolve the scratch address (this
// loads the module that holds it) and load the DHT kernels.
static void* scratch_for_current_device()
{
    int dev = -1;
    SKL_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices)
        fail(SKL_ERR_INVALID, "skl_dht_device_noalloc: device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        SKL_CUDA(cudaGetSymbolAddress(&p, g_dht_scratch));
        dht_load_kernels();
        g_scratch_ptr[dev] = p;
    }
    return g_scratch_ptr[dev];
}

// Forget the per-device addresses (skl_finalize): a device reset destroys
// the context they belong to.
void noalloc_forget_scratch()
{
    std::lock_guard<std::mutex> lk(g_setup_mu);
    for (auto& p : g_scratch_ptr) p = nullptr;
}

template <typename T>
static void dht_noalloc(const double* A, int64_t lda, int64_t n, int64_t d, const double* D,
                        int64_t N, double* Y, int64_t ldy, cudaStream_t st)
{
    void* scr = scratch_for_current_device();
    dht_hash<T>(A, lda, n, d, D, N, nullptr, nullptr, 1, 0, (T*)nullptr, 0, Y, ldy, scr,
                kDhtNoallocScratchBytes, st);
    SKL_CUDA(cudaGetLastError());
}

}  // namespace skl

using namespace skl;

namespace {
struct DhtArgs {
    const double* A;
    int64_t lda, n, d;
    const double* D;
    int64_t N;
    int precision;
    double* Y;
    int64_t ldy;
    void* stream;
};

void run_dht_noalloc(void* p)
{
    const DhtArgs& a = *(const DhtArgs*)p;
    if (!a.A || !a.D || !a.Y || a.n <= 0 || a.d <= 0 || a.lda < a.n || a.N < a.n ||
        a.ldy < a.N)
        fail(SKL_ERR_INVALID, "skl_dht_device_noalloc: bad argument");
    if (a.N > (int64_t)SKL_DHT_NOALLOC_MAX_N)
        fail(SKL_ERR_INVALID,
             "skl_dht_device_noalloc: N = " + std::to_string(a.N) +
                 " exceeds the static scratch limit N <= " +
                 std::to_string((long long)SKL_DHT_NOALLOC_MAX_N) +
                 "; use skl_dht or the solvers for longer transforms");
    if (a.d > INT32_MAX) fail(SKL_ERR_INVALID, "skl_dht_device_noalloc: d too large");
    cudaStream_t st = (cudaStream_t)a.stream;
    if (a.precision == SKL_PREC_FP64)
        dht_noalloc<double>(a.A, a.lda, a.n, a.d, a.D, a.N, a.Y, a.ldy, st);
    else
        dht_noalloc<float>(a.A, a.lda, a.n, a.d, a.D, a.N, a.Y, a.ldy, st);
}
}  // namespace

extern "C" skl_status skl_dht_device_noalloc(const double* A, int64_t lda, int64_t n, int64_t d,
                                             const double* D, int64_t N, int precision,
                                             double* Y, int64_t ldy, void* stream)
{
    DhtArgs a{A, lda, n, d, D, N, precision, Y, ldy, stream};
    return run_guarded(run_dht_noalloc, &a);
}
