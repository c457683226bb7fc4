// skl_api.cpp -- C ABI entry points and the solve pipelines.
//
// Sparse pipeline (ls_sparse_spqr, src/ls_sparse_spqr.cpp:79-214):
//   upload + validate CSC, CSR copy                    (device)
//   hash stream (glibc-compatible, bit-exact)          (host thread, overlapped)
//   SA = S*A (equilibrated), Sb = S*b                  k_sketch.cu
//   randomized CPQR of SA, c = Q^T Sb                  k_qr.cu
//   rank (relative |R_ii| rule), M = R11^{-1}, rcond   k_trinv.cu
//   xs = D P1 M c, r_s = b - A xs, early exit          k_lsqr.cu
//   LSQR on A P1 D M from r_s, x = D P1 M (c + y)      k_lsqr.cu
//   FP64 residual / backward error, optional restarts
// Dense pipeline (ls_dense_hashing_blendenpik, src/ls_dense_hashing_blendenpik.cpp:23-149)
// follows the same steps with the DHT-hashing sketch and dense products.
#include <algorithm>
#include <array>
#include <chrono>
#include <map>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <mutex>
#include <thread>
#include <atomic>
#include <condition_variable>
#include <type_traits>
#include <vector>

#include "skl_internal.hpp"

namespace skl {

// Upper bound on the refinement steps of the mixed path's sketch solution
// (SKILLS_SKETCH_REFINE=<n>; 0 disables).
static int sketch_refine_max_steps()
{
    static const int v = [] {
        const char* e = std::getenv("SKILLS_SKETCH_REFINE");
        return e ? std::max(0, std::atoi(e)) : 6;
    }();
    return v;
}

// ------------------------------------------------------------- errors ----
static thread_local std::string t_last_error;
static thread_local int64_t t_launches = 0;

void fail(skl_status s, const std::string& msg) { throw Error(s, msg); }

void check_cuda(cudaError_t e, const char* what, const char* file, int line)
{
    if (e != cudaSuccess) {
        char buf[512];
        snprintf(buf, sizeof buf, "CUDA error %s (%d) in %s at %s:%d", cudaGetErrorString(e),
                 (int)e, what, file, line);
        throw Error(SKL_ERR_CUDA, buf);
    }
}

static int trace_enabled()
{
    static const int v = [] {
        const char* e = std::getenv("SKILLS_TRACE");
        return (e && e[0] == '1') ? 1 : 0;
    }();
    return v;
}

void allow_max_dynamic_smem(const void* fn)
{
    int dev = 0, optin = 0;
    SKL_CUDA(cudaGetDevice(&dev));
    SKL_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    cudaFuncAttributes fa;
    SKL_CUDA(cudaFuncGetAttributes(&fa, fn));
    SKL_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  optin - (int)fa.sharedSizeBytes));
}

// Phase boundary: a launch that failed (bad configuration) is reported here
// instead of letting later phases run on unwritten buffers.  With
// SKILLS_TRACE=1 also synchronises and prints the phase.
void trace_phase(cudaStream_t st, const char* name)
{
    SKL_CUDA(cudaPeekAtLastError());
    if (!trace_enabled()) return;
    static auto t0 = std::chrono::steady_clock::now();
    cudaError_t e = cudaStreamSynchronize(st);
    double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    fprintf(stderr, "[skl] %10.3f ms  %s  (%s)\n", ms, name, cudaGetErrorString(e));
    fflush(stderr);
}

void note_launch() { ++t_launches; }
int64_t launches_since_reset() { return t_launches; }
void reset_launch_count() { t_launches = 0; }

template <typename F>
static skl_status guarded(F&& fn)
{
    try {
        t_last_error.clear();
        fn();
        return SKL_OK;
    } catch (const Error& e) {
        t_last_error = e.what();
        return e.status;
    } catch (const std::bad_alloc&) {
        t_last_error = "host allocation failed";
        return SKL_ERR_ALLOC;
    } catch (const std::exception& e) {
        t_last_error = e.what();
        return SKL_ERR_INVALID;
    }
}

skl_status run_guarded(void (*fn)(void*), void* arg)
{
    return guarded([&] { fn(arg); });
}

// -------------------------------------------------------------- arena ----
void Arena::reserve(size_t bytes)
{
    if (bytes <= cap_) return;
    release();
    bytes = (bytes + ((size_t)1 << 20) - 1) & ~(((size_t)1 << 20) - 1);
    cudaError_t e = cudaMalloc((void**)&base_, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        base_ = nullptr;
        fail(SKL_ERR_ALLOC, "device allocation of " + std::to_string(bytes >> 20) + " MiB failed");
    }
    cap_ = bytes;
    used_ = 0;
}

void* Arena::take(size_t bytes)
{
    size_t b = (bytes + 255) & ~(size_t)255;
    if (used_ + b > cap_) fail(SKL_ERR_ALLOC, "arena exhausted (internal sizing error)");
    void* p = base_ + used_;
    used_ += b;
    return p;
}

void Arena::release()
{
    if (base_) cudaFree(base_);
    base_ = nullptr;
    cap_ = used_ = 0;
}

// ------------------------------------------------------------ contexts ----
static std::mutex g_ctx_mu;
static std::vector<std::vector<Context*>> g_ctx;   // [device][slot]

Context& context(int device, int slot)
{
    std::lock_guard<std::mutex> lk(g_ctx_mu);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        fail(SKL_ERR_NO_DEVICE, "no CUDA device available");
    }
    if (device < 0 || device >= ndev) fail(SKL_ERR_INVALID, "device ordinal out of range");
    if ((int)g_ctx.size() < ndev) g_ctx.resize(ndev);
    if ((int)g_ctx[device].size() <= slot) g_ctx[device].resize(slot + 1, nullptr);
    SKL_CUDA(cudaSetDevice(device));
    if (!g_ctx[device][slot]) {
        cudaDeviceProp prop;
        SKL_CUDA(cudaGetDeviceProperties(&prop, device));
        if (prop.major != 10)
            fail(SKL_ERR_NO_DEVICE, std::string("device is not a Blackwell sm_10x part: ") + prop.name);
        Context* c = new Context();
        c->device = device;
        SKL_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        for (auto& e : c->ev) SKL_CUDA(cudaEventCreate(&e));
        SKL_CUDA(cudaMalloc((void**)&c->dev_status, 256));
        SKL_CUDA(cudaMemset(c->dev_status, 0, 256));
        c->host_pinned_bytes = 4096;
        SKL_CUDA(cudaMallocHost(&c->host_pinned, c->host_pinned_bytes));
        g_ctx[device][slot] = c;
    }
    return *g_ctx[device][slot];
}

void release_all_contexts()
{
    std::lock_guard<std::mutex> lk(g_ctx_mu);
    for (size_t d = 0; d < g_ctx.size(); ++d) {
        for (Context*& c : g_ctx[d]) {
            if (!c) continue;
            cudaSetDevice((int)d);
            cudaStreamSynchronize(c->stream);
            c->arena.release();
            c->staging.release();
            for (auto& e : c->ev) cudaEventDestroy(e);
            cudaFree(c->dev_status);
            cudaFreeHost(c->host_pinned);
            cudaStreamDestroy(c->stream);
            delete c;
            c = nullptr;
        }
    }
}

// ------------------------------------------------------------- helpers ---
static float elapsed(cudaEvent_t a, cudaEvent_t b)
{
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

static int64_t round_up(int64_t x, int64_t q) { return (x + q - 1) / q * q; }

static void check_opts(const skl_opts& o)
{
    if (!(o.gamma > 0.0) || !std::isfinite(o.gamma)) fail(SKL_ERR_INVALID, "gamma must be > 0");
    if (o.k < 1) fail(SKL_ERR_INVALID, "k must be >= 1");
    if (o.max_it < 0) fail(SKL_ERR_INVALID, "max_it must be >= 0");
    if (o.precision != SKL_PREC_MIXED && o.precision != SKL_PREC_FP64)
        fail(SKL_ERR_INVALID, "unknown precision");
}

// ------------------------------------------------------------ autotuning --
// opts.autotune = 1: the first solve of a shape class times the candidates of
// each tunable launch shape on its own data -- the sketch's block size, the
// CPQR's panel width (whole factorizations of a copy of the sketch), the lanes
// per row / column of LSQR's two sparse products -- and caches the fastest
// for the process (skl_finalize clears the cache).  Shape class: precision
// and half-octave buckets of n, d, nnz per row and m.
struct Tuned {
    int sketch_threads = 0, nb = 0, lanes_n = 0, lanes_t = 0;
};
static std::mutex g_tune_mu;
static std::map<std::array<int, 5>, Tuned> g_tune;

static int octave_bucket(double x) { return (int)std::lround(2.0 * std::log2(std::max(x, 1.0))); }

static std::array<int, 5> tune_key(int prec, int64_t n, int64_t d, int64_t nnz, int64_t m)
{
    return {prec, octave_bucket((double)n), octave_bucket((double)d),
            octave_bucket(16.0 * (double)nnz / (double)std::max<int64_t>(n, 1)), octave_bucket((double)m)};
}

void tune_cache_clear()
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune.clear();
}

// Median of three timed runs of fn on st after one warm-up.
template <typename F>
static float time_median3(cudaStream_t st, F&& fn)
{
    cudaEvent_t e0, e1;
    SKL_CUDA(cudaEventCreate(&e0));
    SKL_CUDA(cudaEventCreate(&e1));
    fn();
    float t[3];
    for (float& v : t) {
        SKL_CUDA(cudaEventRecord(e0, st));
        fn();
        SKL_CUDA(cudaEventRecord(e1, st));
        SKL_CUDA(cudaEventSynchronize(e1));
        SKL_CUDA(cudaEventElapsedTime(&v, e0, e1));
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    std::sort(t, t + 3);
    return t[1];
}

// Status bit a QR pivot selection sets when it meets non-finite values.
constexpr unsigned kQrSelectBit = 8u;

static unsigned read_status(Context& C, cudaStream_t st)
{
    unsigned v = 0;
    SKL_CUDA(cudaMemcpyAsync(C.host_pinned, C.dev_status, sizeof(unsigned), cudaMemcpyDeviceToHost,
                             st));
    SKL_CUDA(cudaStreamSynchronize(st));
    v = *(unsigned*)C.host_pinned;
    return v;
}

// Device-resident inputs of a sparse solve after upload/validation.
struct SparseDev {
    int64_t n, d, nnz;
    const int64_t* Ap; const int64_t* Ai; const double* Ax; const double* b;
};

// ------------------------------------------------------- sparse solve ---
template <typename T>
static void sparse_pipeline(Context& C, cudaStream_t st, const SparseDev& in, double* x_dev,
                            const skl_opts& o, skl_info& info, bool timing_upload,
                            std::thread* hash_thread, std::vector<uint32_t>* host_hidx)
{
    const int64_t n = in.n, d = in.d, nnz = in.nnz;
    const int64_t k = o.k;
    const int64_t m = (int64_t)std::ceil((double)d * o.gamma);
    if (k > m) fail(SKL_ERR_INVALID, "k exceeds the sketch size m = ceil(gamma*d)");
    if (m > 0x7fffffff || nnz > 0x7fffffff || n > 0x7fffffff)
        fail(SKL_ERR_INVALID, "problem too large for 32-bit device indices");
    const bool mixed = std::is_same<T, float>::value;
    const int64_t ld = round_up(m, 32);
    const int64_t mn = std::min(m, d);
    info.sketch_rows = m;

    // ---- workspace layout (sized once, then carved) ----
    const size_t qr_ws = cpqr_workspace_bytes<T>(m, d);
    const size_t inv_ws = trinv_workspace_bytes<T>(d) + (size_t)d * d * sizeof(T);
    LsqrProblem Pq;
    Pq.n = n; Pq.d = d; Pq.nnz = nnz; Pq.r = d; Pq.precision = o.precision;
    const size_t lsqr_ws = lsqr_workspace_bytes(Pq);
    const size_t csr_scr = build_csr_scratch_ints(n, nnz) * sizeof(int);
    const size_t bkt_scr = build_buckets_scratch_ints(m, n * k) * sizeof(int);
    Sizer S;
    S.add<int>(d + 1); S.add<int>(nnz); S.add<int>(n + 1); S.add<int>(nnz); S.add<double>(nnz);
    S.add<char>(mixed ? (int64_t)(2 * nnz * sizeof(float2)) : 0);
    S.add<unsigned>(n * k); S.add<int>(m + 1); S.add<unsigned>(n * k);
    S.add<T>(ld * d); S.add<double>(d); S.add<double>(d); S.add<double>(m);
    S.add<int>(d); S.add<T>(mn); S.add<int>(4);
    S.add<T>(round_up(d, 4) * d); S.add<T>(round_up(d, 4) * d); S.add<double>(4);
    S.add<double>(d); S.add<double>(n); S.add<double>(d); S.add<double>(1024); S.add<double>(8);
    S.add<char>((int64_t)std::max({qr_ws, inv_ws, lsqr_ws, csr_scr, bkt_scr}));
    S.add<float2>(d);
    S.add<double>(m);
    C.arena.reserve(S.bytes());
    C.arena.reset();
    Arena& Ar = C.arena;
    int* cp = Ar.alloc<int>(d + 1);
    int* ri = Ar.alloc<int>(nnz);
    int* rp = Ar.alloc<int>(n + 1);
    int* ci = Ar.alloc<int>(nnz);
    double* cx = Ar.alloc<double>(nnz);
    float2* cx2 = mixed ? (float2*)Ar.take(nnz * sizeof(float2)) : nullptr;
    float2* rx2 = mixed ? (float2*)Ar.take(nnz * sizeof(float2)) : nullptr;
    unsigned* hidx = Ar.alloc<unsigned>(n * k);
    int* bptr = Ar.alloc<int>(m + 1);
    unsigned* bent = Ar.alloc<unsigned>(n * k);
    T* SA = Ar.alloc<T>(ld * d);
    double* colnorm = Ar.alloc<double>(d);
    double* colscale = Ar.alloc<double>(d);
    double* cvec = Ar.alloc<double>(m);
    int* jpvt = Ar.alloc<int>(d);
    T* tau = Ar.alloc<T>(mn);
    int* dint = Ar.alloc<int>(4);
    T* Mc = Ar.alloc<T>(round_up(d, 4) * d);
    T* Mr = Ar.alloc<T>(round_up(d, 4) * d);
    double* norms = Ar.alloc<double>(4);
    double* yv = Ar.alloc<double>(d);
    double* rs = Ar.alloc<double>(n);
    double* xacc = Ar.alloc<double>(d);
    double* part = Ar.alloc<double>(1024);
    double* scal = Ar.alloc<double>(8);
    void* work = Ar.take(std::max({qr_ws, inv_ws, lsqr_ws, csr_scr, bkt_scr}));
    float2* ysplit = Ar.alloc<float2>(d);
    double* gm = Ar.alloc<double>(m);   // S r_s during the sketch-solution refinement

    cudaEvent_t* ev = C.ev;
    SKL_CUDA(cudaEventRecord(ev[1], st));
    // ---- validate + narrow + CSR ----
    SKL_CUDA(cudaMemsetAsync(C.dev_status, 0, sizeof(unsigned), st));
    csc_narrow(in.Ap, in.Ai, in.Ax, n, d, nnz, cp, ri, C.dev_status, st);
    build_csr(cp, ri, in.Ax, n, d, nnz, rp, ci, cx, (int*)work, st);
    // ---- hash stream (host) -> device buckets ----
    if (hash_thread) hash_thread->join();
    if (!host_hidx || (int64_t)host_hidx->size() != n * k)
        fail(SKL_ERR_INVALID, "hash stream missing for the sparse sketch");
    SKL_CUDA(cudaMemcpyAsync(hidx, host_hidx->data(), n * k * sizeof(unsigned),
                             cudaMemcpyHostToDevice, st));
    check_hash_rows(hidx, n * k, m, C.dev_status, st);
    unsigned bad = read_status(C, st);
    if (bad & 1u) fail(SKL_ERR_INVALID, "CSC column pointers are not a valid structure");
    if (bad & 2u) fail(SKL_ERR_INVALID, "CSC row index out of range");
    if (bad & 4u) fail(SKL_ERR_NONFINITE, "A contains NaN or Inf");
    if (bad & 16u) fail(SKL_ERR_INVALID, "hash row index out of range");
    trace_phase(st, "csr+validate");
    build_buckets(hidx, n, (int)k, m, bptr, bent, (int*)work, st);
    trace_phase(st, "buckets");
    SKL_CUDA(cudaEventRecord(ev[2], st));
    // ---- launch shapes: the tuned ones of this shape class, or tune now ----
    Tuned tuned;
    const auto tkey = tune_key(o.precision, n, d, nnz, m);
    bool have_tuned = false;
    if (o.autotune) {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune.find(tkey);
        if (it != g_tune.end()) {
            tuned = it->second;
            have_tuned = true;
        }
    }
    const bool tuning = o.autotune && !have_tuned;
    // ---- sketch ----
    if (tuning) {
        float best = 1e30f;
        for (int th : {256, 512, 1024}) {
            const float t = time_median3(st, [&] {
                sketch_sparse<T>(cp, ri, in.Ax, n, d, hidx, (int)k, m, SA, ld, 1, colnorm, colscale, st, th);
            });
            if (t < best) {
                best = t;
                tuned.sketch_threads = th;
            }
        }
    }
    sketch_sparse<T>(cp, ri, in.Ax, n, d, hidx, (int)k, m, SA, ld, 1, colnorm, colscale, st,
                     tuned.sketch_threads);
    sketch_rhs(bptr, bent, m, (int)k, in.b, cvec, st);
    if (mixed) {
        // LSQR's float pairs hold the equilibrated values A(:, c) / ||A(:, c)||:
        // |value| <= 1, so no finite input overflows the float range
        split_csr_scaled(ci, cx, nnz, colscale, cx2, st);
        split_csc_scaled(cp, in.Ax, d, colscale, rx2, st);
    }
    trace_phase(st, "sketch");
    SKL_CUDA(cudaEventRecord(ev[3], st));
    // ---- randomized CPQR, c = Q^T S b ----
    if (tuning && mixed) {
        // whole factorizations of a copy of the sketch at each panel width
        T* SAc = nullptr;
        double* cc = nullptr;
        SKL_CUDA(cudaMallocAsync((void**)&SAc, (size_t)ld * d * sizeof(T), st));
        SKL_CUDA(cudaMallocAsync((void**)&cc, (size_t)m * sizeof(double), st));
        float best = 1e30f;
        int last_nb = 0;
        for (int cap : {64, 48, 32}) {
            const int nbw = cpqr_panel_width(m, d, cap);
            if (nbw == last_nb) continue;
            last_nb = nbw;
            const float t = time_median3(st, [&] {
                SKL_CUDA(cudaMemcpyAsync(SAc, SA, (size_t)ld * d * sizeof(T), cudaMemcpyDeviceToDevice, st));
                SKL_CUDA(cudaMemcpyAsync(cc, cvec, (size_t)m * sizeof(double), cudaMemcpyDeviceToDevice, st));
                cpqr<T>(SAc, m, d, ld, jpvt, tau, work, C.dev_status, st, cc, 1, nullptr, nbw);
            });
            if (t < best) {
                best = t;
                tuned.nb = nbw;
            }
        }
        SKL_CUDA(cudaFreeAsync(SAc, st));
        SKL_CUDA(cudaFreeAsync(cc, st));
        SKL_CUDA(cudaMemsetAsync(C.dev_status, 0, sizeof(unsigned), st));
    }
    cpqr<T>(SA, m, d, ld, jpvt, tau, work, C.dev_status, st, cvec, 1,
            o.profile ? info.qr_prof_ms : nullptr, tuned.nb);
    {
        const unsigned qs = read_status(C, st);
        if (qs & kStatusTcTimeout) fail(SKL_ERR_TIMEOUT, "a kernel's bounded wait gave up (tensor-core product or sample QRP exchange)");
        if (qs & kQrSelectBit) fail(SKL_ERR_NONFINITE, "non-finite values in the sketch factorization");
    }
    trace_phase(st, "cpqr");
    SKL_CUDA(cudaEventRecord(ev[4], st));
    // ---- rank, inverse, condition ----
    // FP64: SPQR's default tolerance 20 (m + d) eps relative to the largest
    // (equilibrated) column.  FP32: an exactly dependent column leaves |R_ii|
    // of up to ~sqrt(m) eps_32 |R_00| (measured: 1.6e-6 at m = 8,500), so the
    // factorization resolves nothing below 2 sqrt(m) eps_32.  Columns under
    // that bound are not dropped: they stay in LSQR's basis with unit
    // preconditioning (M extended by an identity block), and the FP64-class
    // iteration decides whether they reduce the residual, as an FP64
    // factorization would have.  Exactly dependent ones cost nothing there
    // (their gradient is a combination of the resolved columns' gradients).
    double rel = o.rank_tol;
    const bool carry_unresolved = mixed && !(rel > 0.0);
    if (!(rel > 0.0))
        rel = mixed ? 2.0 * std::sqrt((double)m) * 5.960464477539063e-08
                    : 20.0 * (double)(m + d) * 2.220446049250313e-16;
    int64_t rank = count_rank<T>(SA, ld, mn, 0.0, rel, dint, (int*)C.host_pinned, st);
    if (rank == 0) fail(SKL_ERR_RANK_ZERO, "SPQR Factorization fails");
    info.rank = rank;
    const int64_t rank_lsqr = carry_unresolved ? mn : rank;
    info.unresolved_cols = rank_lsqr - rank;
    const int64_t ldm = round_up(rank_lsqr, 4);   // 16-byte aligned rows/columns of M
    trinv_upper<T>(SA, ld, rank, 0.0, Mc, ldm, norms, work, st);
    SKL_CUDA(cudaMemcpyAsync(C.host_pinned, norms, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
    SKL_CUDA(cudaStreamSynchronize(st));
    double nr = ((double*)C.host_pinned)[0], nm = ((double*)C.host_pinned)[1];
    double rcond = (nr > 0 && nm > 0) ? 1.0 / (nr * nm) : 0.0;
    info.rcond_r11 = rcond;
    info.success = rcond > o.rcond_threshold ? 1 : 0;
    if (!info.success && o.perturb != 0.0) {
        trinv_upper<T>(SA, ld, rank, o.perturb, Mc, ldm, norms, work, st);
    }
    extend_identity<T>(Mc, ldm, rank, rank_lsqr, st);
    transpose_upper<T>(Mc, ldm, rank_lsqr, Mr, st);
    trace_phase(st, "rank+inverse");
    LsqrProblem P;
    P.n = n; P.d = d; P.nnz = nnz;
    P.rp = rp; P.ci = ci; P.cx = mixed ? (const void*)cx2 : (const void*)cx;
    P.cp = cp; P.ri = ri; P.rx = mixed ? (const void*)rx2 : (const void*)in.Ax;
    P.cx64 = cx; P.rx64 = in.Ax;
    P.cols = jpvt; P.colscale = colscale;
    P.opscale = mixed ? nullptr : colscale;   // the float pairs are already equilibrated
    P.M = Mc; P.Mrow = Mr; P.ldm = ldm; P.r = rank; P.precision = o.precision;
    if (tuning) {
        P.r = rank_lsqr;
        tune_lsqr_products(P, work, st);   // the workspace is idle between the inverse and LSQR
        P.r = rank;
        tuned.lanes_n = P.lanes_n;
        tuned.lanes_t = P.lanes_t;
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune[tkey] = tuned;
    } else {
        P.lanes_n = tuned.lanes_n;
        P.lanes_t = tuned.lanes_t;
    }
    info.tuned[0] = tuned.sketch_threads;
    info.tuned[1] = mixed ? cpqr_panel_width(m, d, tuned.nb) : 0;   // the width the FP32 CPQR used
    info.tuned[2] = tuned.lanes_n;
    info.tuned[3] = tuned.lanes_t;
    // ---- explicit sketch solution xs = D P1 M c (resolved columns only) ----
    SKL_CUDA(cudaMemsetAsync(x_dev, 0, d * sizeof(double), st));
    precond_apply(P, cvec, x_dev, ysplit, st);
    residual_and_backward(P, x_dev, in.b, rs, part, scal, st);
    trace_phase(st, "explicit solution");
    SKL_CUDA(cudaMemcpyAsync(C.host_pinned, scal, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
    SKL_CUDA(cudaStreamSynchronize(st));
    double rnorm = ((double*)C.host_pinned)[0];
    if (mixed && !(rnorm < o.abs_tol)) {
        // The reference forms x_s from an FP64 factorization; an FP32 one leaves
        // x_s ~eps32*cond(R) off the sketched solution, and LSQR would spend
        // iterations removing that consistent part of r_s.  Refine c against
        // the FP64 residual while a step is predicted to shrink ||r_s|| by at
        // least 13 %: the correction dc = Q1^T S r_s removes the part of the
        // sketched residual in range(S A), so ||r_s'|| ~ ||S r_s|| *
        // sqrt(1 - (||dc|| / ||S r_s||)^2).  Refinement is not stopped merely by
        // ||r_s|| < abs_tol: the early exit must see an x_s as good as the
        // reference's.
        const int steps = sketch_refine_max_steps();
        double* h = (double*)work;   // n doubles; the workspace is idle here
        double* hp = (double*)C.host_pinned;
        bool refined = false;
        for (int s = 0; s < steps; ++s) {
            sketch_refine_direction(P, bptr, bent, hidx, (int)k, m, rs, gm, h, xacc, yv, part,
                                    scal + 2, st);
            SKL_CUDA(cudaMemcpyAsync(hp, scal + 2, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
            SKL_CUDA(cudaStreamSynchronize(st));
            if (!(hp[1] >= 0.5 * hp[0])) break;
            sketch_refine_apply(P, 1.0, yv, cvec, in.b, x_dev, rs, part, scal + 4, st);
            SKL_CUDA(cudaMemcpyAsync(hp, scal + 4, sizeof(double), cudaMemcpyDeviceToHost, st));
            SKL_CUDA(cudaStreamSynchronize(st));
            const double rn = hp[0];
            if (!(rn < rnorm)) {
                // no progress (cond(R) too large for the FP32 factor): undo the step
                sketch_refine_apply(P, -1.0, yv, cvec, in.b, x_dev, rs, part, scal + 4, st);
                break;
            }
            rnorm = rn;
            refined = true;
            ++info.sketch_refine_steps;
        }
        if (refined) residual_and_backward(P, x_dev, in.b, rs, part, scal, st);
        // host_pinned[0..1] = ||r_s||, ||A^T r_s|| again for the checks below
        SKL_CUDA(cudaMemcpyAsync(hp, scal, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
        SKL_CUDA(cudaStreamSynchronize(st));
        rnorm = hp[0];
        trace_phase(st, "sketch refinement");
    }
    SKL_CUDA(cudaEventRecord(ev[5], st));
    info.explicit_residual = rnorm;
    info.it = 0;
    info.flag = 0;
    // ||A||_F from the column norms
    double fro = 0.0;
    {
        std::vector<double> cn((size_t)d);
        SKL_CUDA(cudaMemcpyAsync(cn.data(), colnorm, d * sizeof(double), cudaMemcpyDeviceToHost, st));
        SKL_CUDA(cudaStreamSynchronize(st));
        for (double v : cn) fro += v * v;
        fro = std::sqrt(fro);
    }
    double be = (rnorm > 0 && fro > 0) ? ((double*)C.host_pinned)[1] / (fro * rnorm) : 0.0;
    if (!(rnorm < o.abs_tol)) {
        // ---- LSQR from r_s; x = x_s + D P1 M y (src/ls_sparse_spqr.cpp:181-208) ----
        // The correction is added to the same rounded x_s that r_s was formed
        // from: LSQR compensates x_s's rounding, and D P1 M (c + y) recomputed
        // in one product would re-round it with cond(R) amplification (on the
        // 120,000 x 5,000 workload that left ||b - A x|| 1.4e-3 relative above
        // the minimum and the backward error at 2.3e-3 instead of 3.4e-4).
        P.r = rank_lsqr;
        int64_t total_it = 0;
        int flag = 1;
        int64_t restarts = 0;
        const double btol = o.backward_tol;
        // first solve
        auto add_prof = [&](const LsqrResult& Rr) {
            for (int q = 0; q < 4; ++q) {
                info.prof_ms[q] += Rr.prof_ms[q];
                info.prof_launches[q] += Rr.prof_launches[q];
            }
        };
        LsqrResult R = lsqr_run(P, rs, o.it_tol, o.max_it, yv, work, C.dev_status, C.host_pinned,
                                st, o.profile, C.stream);
        add_prof(R);
        total_it += R.it;
        flag = R.flag;
        SKL_CUDA(cudaMemsetAsync(xacc, 0, d * sizeof(double), st));
        precond_apply(P, yv, xacc, ysplit, st);
        vec_add(x_dev, xacc, d, st);
        residual_and_backward(P, x_dev, in.b, rs, part, scal, st);
        SKL_CUDA(cudaMemcpyAsync(C.host_pinned, scal, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
        SKL_CUDA(cudaStreamSynchronize(st));
        rnorm = ((double*)C.host_pinned)[0];
        be = (rnorm > 0 && fro > 0) ? ((double*)C.host_pinned)[1] / (fro * rnorm) : 0.0;
        // restarts from the FP64 residual while the backward error target is missed
        while (btol > 0.0 && be > btol && restarts < o.max_refine && total_it < o.max_it) {
            ++restarts;
            R = lsqr_run(P, rs, o.it_tol, o.max_it - total_it, yv, work, C.dev_status, C.host_pinned,
                         st, o.profile, C.stream);
            add_prof(R);
            total_it += R.it;
            flag = R.flag;
            SKL_CUDA(cudaMemsetAsync(xacc, 0, d * sizeof(double), st));
            precond_apply(P, yv, xacc, ysplit, st);
            vec_add(x_dev, xacc, d, st);
            residual_and_backward(P, x_dev, in.b, rs, part, scal, st);
            SKL_CUDA(cudaMemcpyAsync(C.host_pinned, scal, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
            SKL_CUDA(cudaStreamSynchronize(st));
            rnorm = ((double*)C.host_pinned)[0];
            be = (rnorm > 0 && fro > 0) ? ((double*)C.host_pinned)[1] / (fro * rnorm) : 0.0;
        }
        info.it = total_it;
        info.flag = flag;
    }
    SKL_CUDA(cudaEventRecord(ev[6], st));
    SKL_CUDA(cudaEventSynchronize(ev[6]));
    info.residual_norm = rnorm;
    info.backward_error = be;
    info.t_setup_ms = elapsed(ev[1], ev[2]);
    info.t_sketch_ms = elapsed(ev[2], ev[3]);
    info.t_qr_ms = elapsed(ev[3], ev[4]);
    info.t_precond_ms = elapsed(ev[4], ev[5]);
    info.t_lsqr_ms = elapsed(ev[5], ev[6]);
    info.t_total_ms = elapsed(timing_upload ? ev[0] : ev[1], ev[6]);
    if (timing_upload) info.t_upload_ms = elapsed(ev[0], ev[1]);
    unsigned stt = read_status(C, st);
    if (stt & 1u) fail(SKL_ERR_TIMEOUT, "a bounded device wait gave up");
}

static void fill_default(skl_opts* o)
{
    std::memset(o, 0, sizeof(*o));
    o->gamma = 1.1;
    o->k = 3;
    o->abs_tol = 1e-8;
    o->it_tol = 1e-6;
    o->max_it = 10000;
    o->rcond_threshold = 1e-10;
    o->perturb = 1e-10;
    o->rcond = 1e-10;
    o->rank_tol = 0.0;
    o->precision = SKL_PREC_MIXED;
    o->use_cpqr = 1;
    o->seed_mode = 0;
    o->seed = 0;
    o->wisdom = 0;
    o->backward_tol = 0.0;
    o->max_refine = 3;
    o->device = 0;
    o->autotune = 0;
}

static void validate_csc_header(const skl_csc* A)
{
    if (!A) fail(SKL_ERR_INVALID, "A is null");
    if (A->m < 0 || A->n < 0) fail(SKL_ERR_INVALID, "negative dimension");
    if (A->n > 0 && (!A->p)) fail(SKL_ERR_INVALID, "A->p is null");
    if (A->m < A->n) fail(SKL_ERR_NOT_OVERDETERMINED, "Matrix is not overdetermined.");
}

// One sparse solve on context C and stream st.  The hash stream arrives
// either from a worker thread still filling hh (single solves overlap it with
// the upload and validation) or already filled (th = nullptr).
static void sparse_solve_core(Context& C, cudaStream_t st, const skl_csc* A, const double* b,
                              double* x, const skl_opts& o, skl_info& inf, bool host,
                              std::thread* th, std::vector<uint32_t>* hh)
{
    const int64_t n = A->m, d = A->n;
    SparseDev in;
    in.n = n;
    in.d = d;
    int64_t nnz = 0;
    SKL_CUDA(cudaEventRecord(C.ev[0], st));
    if (host) {
        if (!A->p) fail(SKL_ERR_INVALID, "A->p is null");
        nnz = A->p[d];
        if (nnz < 0) fail(SKL_ERR_INVALID, "negative nnz");
        if (nnz > 0 && (!A->i || !A->x)) fail(SKL_ERR_INVALID, "A->i or A->x is null");
        Sizer S;
        S.add<int64_t>(d + 1); S.add<int64_t>(nnz); S.add<double>(nnz); S.add<double>(n);
        S.add<double>(d);
        C.staging.reserve(S.bytes());
        C.staging.reset();
        int64_t* Ap = C.staging.alloc<int64_t>(d + 1);
        int64_t* Ai = C.staging.alloc<int64_t>(nnz);
        double* Ax = C.staging.alloc<double>(nnz);
        double* bd = C.staging.alloc<double>(n);
        double* xd = C.staging.alloc<double>(d);
        SKL_CUDA(cudaMemcpyAsync(Ap, A->p, (d + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st));
        if (nnz > 0) {
            SKL_CUDA(cudaMemcpyAsync(Ai, A->i, nnz * sizeof(int64_t), cudaMemcpyHostToDevice, st));
            SKL_CUDA(cudaMemcpyAsync(Ax, A->x, nnz * sizeof(double), cudaMemcpyHostToDevice, st));
        }
        SKL_CUDA(cudaMemcpyAsync(bd, b, n * sizeof(double), cudaMemcpyHostToDevice, st));
        in.Ap = Ap; in.Ai = Ai; in.Ax = Ax; in.b = bd; in.nnz = nnz;
        if (o.precision == SKL_PREC_MIXED)
            sparse_pipeline<float>(C, st, in, xd, o, inf, true, th, hh);
        else
            sparse_pipeline<double>(C, st, in, xd, o, inf, true, th, hh);
        SKL_CUDA(cudaMemcpyAsync(x, xd, d * sizeof(double), cudaMemcpyDeviceToHost, st));
        SKL_CUDA(cudaStreamSynchronize(st));
    } else {
        SKL_CUDA(cudaMemcpyAsync(C.host_pinned, A->p + d, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
        SKL_CUDA(cudaStreamSynchronize(st));
        nnz = *(int64_t*)C.host_pinned;
        in.Ap = A->p; in.Ai = A->i; in.Ax = A->x; in.b = b; in.nnz = nnz;
        if (o.precision == SKL_PREC_MIXED)
            sparse_pipeline<float>(C, st, in, x, o, inf, false, th, hh);
        else
            sparse_pipeline<double>(C, st, in, x, o, inf, false, th, hh);
    }
}

static void sparse_solve_common(const skl_csc* A, const double* b, double* x, const skl_opts* opts,
                                skl_info* info, bool host)
{
    skl_opts o;
    if (opts) o = *opts;
    else fill_default(&o);
    check_opts(o);
    validate_csc_header(A);
    if (!b || !x) fail(SKL_ERR_INVALID, "b or x is null");
    skl_info inf;
    std::memset(&inf, 0, sizeof inf);
    const int64_t n = A->m, d = A->n;
    if (d == 0) {
        if (info) *info = inf;
        return;
    }
    Context& C = context(o.device, 0);
    reset_launch_count();
    cudaStream_t st = o.stream ? (cudaStream_t)o.stream : C.stream;
    const int64_t m = (int64_t)std::ceil((double)d * o.gamma);
    if (o.k > m) fail(SKL_ERR_INVALID, "k exceeds the sketch size m = ceil(gamma*d)");
    // host hash stream in a worker thread (serial Fisher-Yates)
    std::vector<uint32_t> hh((size_t)(n * o.k));
    double hash_ms = 0.0;
    std::thread th([&]() {
        auto t0 = std::chrono::steady_clock::now();
        if (o.seed_mode) rng_srand(o.seed);
        rng_lock();
        gen_hash_packed(m, n, o.k, hh.data());
        rng_unlock();
        hash_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    });
    struct Joiner {
        std::thread& t;
        ~Joiner() { if (t.joinable()) t.join(); }
    } joiner{th};
    sparse_solve_core(C, st, A, b, x, o, inf, host, &th, &hh);
    inf.t_host_hash_ms = hash_ms;
    inf.kernel_launches = launches_since_reset();
    if (info) *info = inf;
}

// Batched sparse solves (host buffers): hashing drawn here in problem order,
// exactly as a loop of skl_sparse_solve calls with the same options would draw
// it, then the problems spread over worker threads, each with its own device
// context and stream.
static void batched_sparse_common(int64_t nprob, const skl_csc* A, const double* const* b,
                                  double* const* x, const skl_opts* opts, skl_info* info,
                                  skl_status* status)
{
    if (nprob < 0) fail(SKL_ERR_INVALID, "nprob < 0");
    if (nprob == 0) return;
    if (!A || !b || !x) fail(SKL_ERR_INVALID, "skl_batched_sparse_solve: null array");
    skl_opts o;
    if (opts) o = *opts;
    else fill_default(&o);
    check_opts(o);
    for (int64_t p = 0; p < nprob; ++p) {
        validate_csc_header(&A[p]);
        if (!b[p] || !x[p]) fail(SKL_ERR_INVALID, "skl_batched_sparse_solve: b or x is null");
        if (A[p].n > 0 && o.k > (int64_t)std::ceil((double)A[p].n * o.gamma))
            fail(SKL_ERR_INVALID, "k exceeds the sketch size m = ceil(gamma*d)");
    }
    // hash streams, in problem order, drawn by one producer thread while the
    // workers already solve the problems whose streams are ready (problem p
    // waits for hashed >= p + 1; the producer also releases everyone if it
    // fails, with hash_failed set)
    std::vector<std::vector<uint32_t>> hh((size_t)nprob);
    std::vector<double> hash_ms((size_t)nprob, 0.0);
    std::mutex hash_mu;
    std::condition_variable hash_cv;
    int64_t hashed = 0;
    bool hash_failed = false;
    std::string hash_msg;
    std::thread producer([&] {
        try {
            for (int64_t p = 0; p < nprob; ++p) {
                const int64_t n = A[p].m, d = A[p].n;
                if (d > 0) {
                    const int64_t m = (int64_t)std::ceil((double)d * o.gamma);
                    hh[(size_t)p].resize((size_t)(n * o.k));
                    auto t0 = std::chrono::steady_clock::now();
                    if (o.seed_mode) rng_srand(o.seed);
                    {
                        struct Held {
                            Held() { rng_lock(); }
                            ~Held() { rng_unlock(); }
                        } held;
                        gen_hash_packed(m, n, o.k, hh[(size_t)p].data());
                    }
                    hash_ms[(size_t)p] =
                        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
                }
                {
                    std::lock_guard<std::mutex> lk(hash_mu);
                    hashed = p + 1;
                }
                hash_cv.notify_all();
            }
        } catch (const std::exception& e) {
            std::lock_guard<std::mutex> lk(hash_mu);
            hash_failed = true;
            hash_msg = e.what();
            hashed = nprob;
        }
        hash_cv.notify_all();
    });
    struct ProducerJoin {
        std::thread& t;
        ~ProducerJoin() { if (t.joinable()) t.join(); }
    } producer_join{producer};
    int workers = 8;
    if (const char* e = std::getenv("SKILLS_BATCH_STREAMS")) workers = std::max(1, std::atoi(e));
    workers = (int)std::min<int64_t>(workers, nprob);
    std::atomic<int64_t> next{0};
    std::mutex err_mu;
    skl_status first_status = SKL_OK;
    std::string first_msg;
    auto work = [&](int slot) {
        for (;;) {
            const int64_t p = next.fetch_add(1);
            if (p >= nprob) break;
            skl_info inf;
            std::memset(&inf, 0, sizeof inf);
            skl_status rc = SKL_OK;
            std::string msg;
            bool stream_ok;
            {
                std::unique_lock<std::mutex> lk(hash_mu);
                hash_cv.wait(lk, [&] { return hashed > p; });
                stream_ok = !hash_failed;
            }
            try {
                if (!stream_ok) fail(SKL_ERR_ALLOC, "skl_batched_sparse_solve: hash stream: " + hash_msg);
                if (A[p].n > 0) {
                    Context& C = context(o.device, 1 + slot);
                    reset_launch_count();
                    sparse_solve_core(C, C.stream, &A[p], b[p], x[p], o, inf, true, nullptr,
                                      &hh[(size_t)p]);
                    inf.t_host_hash_ms = hash_ms[(size_t)p];
                    inf.kernel_launches = launches_since_reset();
                }
            } catch (const Error& e) {
                rc = e.status;
                msg = e.what();
            } catch (const std::exception& e) {
                rc = SKL_ERR_CUDA;
                msg = e.what();
            }
            if (info) info[p] = inf;
            if (status) status[p] = rc;
            if (rc != SKL_OK) {
                std::lock_guard<std::mutex> lk(err_mu);
                if (first_status == SKL_OK) {
                    first_status = rc;
                    first_msg = "problem " + std::to_string(p) + ": " + msg;
                }
            }
        }
    };
    std::vector<std::thread> pool;
    for (int w = 0; w < workers; ++w) pool.emplace_back(work, w);
    for (auto& t : pool) t.join();
    producer.join();
    if (first_status != SKL_OK) fail(first_status, first_msg);
}

// --------------------------------------------------------- dense solve ---
// ls_dense_hashing_blendenpik (src/ls_dense_hashing_blendenpik.cpp:23-149),
// with use_cpqr = 0 ls_dense_hashing_blendenpik_noCPQR
// (src/ls_dense_hashing_blendenpik_noCPQR.cpp:23-59), and with sample_rows
// ls_dense_blendenpik (src/ls_dense_blendenpik.cpp:21-70), whose sketch
// rand_subsampled_dct (src/dense_helpers.cpp:42-59) keeps m rows of the
// transform instead of hashing them: hh then holds those m rows, each row its
// own bucket with sign + and k = 1 (so the gather's 1/k is 1), and the rest is
// the noCPQR pipeline.

// Returns false (nothing solved) when the mixed path meets values outside its
// range; the caller then runs the FP64 pipeline.
template <typename T>
static bool dense_pipeline(Context& C, cudaStream_t st, const double* A, int64_t lda, int64_t n,
                           int64_t d, const double* b, double* x_dev, const skl_opts& o,
                           skl_info& info, bool timing_upload, std::thread* host_thread,
                           const std::vector<double>* hD, const std::vector<uint32_t>* hh,
                           int64_t N, bool sample_rows)
{
    const bool mixed = std::is_same<T, float>::value;
    const bool cpqr_on = o.use_cpqr != 0;
    const int64_t k = o.k;
    const int64_t m = (int64_t)std::ceil((double)d * o.gamma);
    if (m < d) fail(SKL_ERR_INVALID, "sketch has fewer rows than A has columns (gamma*d < d)");
    const int64_t ld = round_up(m, 32);
    const int64_t mn = std::min(m, d);
    info.sketch_rows = m;
    const size_t qr_ws = cpqr_workspace_bytes<T>(m, d);
    const size_t inv_ws = trinv_workspace_bytes<T>(d);
    LsqrProblem Pq;
    Pq.n = n; Pq.d = d; Pq.r = d; Pq.precision = o.precision; Pq.Ad = A; Pq.lda = n;
    const size_t lsqr_ws = lsqr_workspace_bytes(Pq);
    const size_t bkt_scr = build_buckets_scratch_ints(m, N * k) * sizeof(int);
    const size_t dht_ws = dht_scratch_bytes(N, o.precision);
    const size_t work_bytes = std::max({qr_ws, inv_ws, lsqr_ws, bkt_scr, dht_ws});
    const int64_t ldm_max = round_up(d, 4);
    Sizer S;
    S.add<double>(n); S.add<unsigned>(N * k); S.add<int>(m + 1); S.add<unsigned>(N * k);
    S.add<char>(mixed ? (int64_t)(n * d * sizeof(float2)) : 0);
    S.add<T>(ld * d); S.add<double>(d); S.add<double>(m); S.add<int>(d); S.add<T>(mn); S.add<int>(4);
    S.add<T>(ldm_max * d); S.add<T>(ldm_max * d); S.add<double>(4); S.add<double>(d);
    S.add<double>(n); S.add<double>(d); S.add<double>(1024); S.add<double>(8);
    S.add<char>((int64_t)work_bytes); S.add<float2>(d);
    C.arena.reserve(S.bytes());
    C.arena.reset();
    Arena& Ar = C.arena;
    double* Dd = Ar.alloc<double>(n);
    unsigned* hidx = Ar.alloc<unsigned>(N * k);
    int* bptr = Ar.alloc<int>(m + 1);
    unsigned* bent = Ar.alloc<unsigned>(N * k);
    float2* A2 = mixed ? (float2*)Ar.take(n * d * sizeof(float2)) : nullptr;
    T* SA = Ar.alloc<T>(ld * d);
    double* colscale = Ar.alloc<double>(d);
    double* cvec = Ar.alloc<double>(m);
    int* jpvt = Ar.alloc<int>(d);
    T* tau = Ar.alloc<T>(mn);
    int* dint = Ar.alloc<int>(4);
    T* Mc = Ar.alloc<T>(ldm_max * d);
    T* Mr = Ar.alloc<T>(ldm_max * d);
    double* norms = Ar.alloc<double>(4);
    double* yv = Ar.alloc<double>(d);
    double* rs = Ar.alloc<double>(n);
    double* xacc = Ar.alloc<double>(d);
    double* part = Ar.alloc<double>(1024);
    double* scal = Ar.alloc<double>(8);
    void* work = Ar.take(work_bytes);
    float2* ysplit = Ar.alloc<float2>(d);
    cudaEvent_t* ev = C.ev;
    SKL_CUDA(cudaEventRecord(ev[1], st));
    if (mixed) {
        SKL_CUDA(cudaMemsetAsync(C.dev_status, 0, sizeof(unsigned), st));
        split_dense(A, lda, n, d, A2, C.dev_status, st);
    }
    {
        std::vector<double> ones((size_t)d, 1.0);
        SKL_CUDA(cudaMemcpyAsync(colscale, ones.data(), d * sizeof(double), cudaMemcpyHostToDevice, st));
        SKL_CUDA(cudaStreamSynchronize(st));
    }
    if (mixed && (read_status(C, st) & kStatusRange)) return false;
    if (host_thread->joinable()) host_thread->join();
    SKL_CUDA(cudaMemcpyAsync(Dd, hD->data(), n * sizeof(double), cudaMemcpyHostToDevice, st));
    if (sample_rows) {
        std::vector<int> bp((size_t)m + 1);
        for (int64_t h = 0; h <= m; ++h) bp[(size_t)h] = (int)h;
        SKL_CUDA(cudaMemcpyAsync(bptr, bp.data(), (m + 1) * sizeof(int), cudaMemcpyHostToDevice, st));
        SKL_CUDA(cudaMemcpyAsync(bent, hh->data(), m * sizeof(unsigned), cudaMemcpyHostToDevice, st));
    } else {
        SKL_CUDA(cudaMemcpyAsync(hidx, hh->data(), N * k * sizeof(unsigned), cudaMemcpyHostToDevice, st));
        build_buckets(hidx, N, (int)k, m, bptr, bent, (int*)work, st);
    }
    SKL_CUDA(cudaEventRecord(ev[2], st));
    // ---- sketch: DHT + hash of A (and b) ----
    dht_hash<T>(A, lda, n, d, Dd, N, bptr, bent, (int)k, m, SA, ld, nullptr, 0, work, work_bytes, st);
    if (cpqr_on) dht_hash_rhs(b, n, Dd, N, bptr, bent, (int)k, m, cvec, work, work_bytes, st);
    trace_phase(st, "dense sketch");
    SKL_CUDA(cudaEventRecord(ev[3], st));
    // ---- QR (pivoted for the CPQR path) ----
    SKL_CUDA(cudaMemsetAsync(C.dev_status, 0, sizeof(unsigned), st));
    cpqr<T>(SA, m, d, ld, jpvt, tau, work, C.dev_status, st, cpqr_on ? cvec : nullptr,
            cpqr_on ? 1 : 0, o.profile ? info.qr_prof_ms : nullptr);
    {
        const unsigned qs = read_status(C, st);
        if (qs & kStatusTcTimeout) fail(SKL_ERR_TIMEOUT, "a kernel's bounded wait gave up (tensor-core product or sample QRP exchange)");
        if (qs & kQrSelectBit) fail(SKL_ERR_NONFINITE, "non-finite values in the sketch factorization");
    }
    trace_phase(st, "dense qr");
    SKL_CUDA(cudaEventRecord(ev[4], st));
    // ---- rank: leading |R_ii| > rcond (absolute, :79-89); noCPQR keeps all ----
    int64_t rank = d;
    if (cpqr_on) {
        // the reference's absolute rule, floored at the working precision's
        // resolution of the sketch (FP32 cannot resolve |R_ii| below eps*|R_00|)
        const double floor_rel = mixed ? 5.960464477539063e-08 : 0.0;
        rank = count_rank<T>(SA, ld, mn, o.rcond, floor_rel, dint, (int*)C.host_pinned, st);
        if (rank == 0) fail(SKL_ERR_RANK_ZERO, "sketch has no diagonal entry above rcond");
    }
    info.rank = rank;
    info.success = 1;
    const int64_t ldm = round_up(rank, 4);
    trinv_upper<T>(SA, ld, rank, 0.0, Mc, ldm, norms, work, st);
    transpose_upper<T>(Mc, ldm, rank, Mr, st);
    SKL_CUDA(cudaMemcpyAsync(C.host_pinned, norms, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
    SKL_CUDA(cudaStreamSynchronize(st));
    {
        double nr = ((double*)C.host_pinned)[0], nm = ((double*)C.host_pinned)[1];
        info.rcond_r11 = (nr > 0 && nm > 0) ? 1.0 / (nr * nm) : 0.0;
    }
    LsqrProblem P;
    P.n = n; P.d = d; P.nnz = n * d;
    P.Ad = mixed ? (const void*)A2 : (const void*)A;
    P.lda = mixed ? n : lda;
    P.Ad64 = A; P.lda64 = lda;
    P.cols = jpvt; P.colscale = colscale;
    P.M = Mc; P.Mrow = Mr; P.ldm = ldm; P.r = rank; P.precision = o.precision;
    // ||A||_F
    fro_partials(A, lda, n, d, part, st);
    std::vector<double> fp(512);
    SKL_CUDA(cudaMemcpyAsync(fp.data(), part, 512 * sizeof(double), cudaMemcpyDeviceToHost, st));
    SKL_CUDA(cudaStreamSynchronize(st));
    double fro = 0.0;
    for (double v : fp) fro += v;
    fro = std::sqrt(fro);
    double rnorm = 0.0, be = 0.0;
    auto residual = [&]() {
        residual_and_backward(P, x_dev, b, rs, part, scal, st);
        SKL_CUDA(cudaMemcpyAsync(C.host_pinned, scal, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
        SKL_CUDA(cudaStreamSynchronize(st));
        rnorm = ((double*)C.host_pinned)[0];
        be = (rnorm > 0 && fro > 0) ? ((double*)C.host_pinned)[1] / (fro * rnorm) : 0.0;
    };
    auto add_prof = [&](const LsqrResult& Rr) {
        for (int q = 0; q < 4; ++q) {
            info.prof_ms[q] += Rr.prof_ms[q];
            info.prof_launches[q] += Rr.prof_launches[q];
        }
    };
    SKL_CUDA(cudaMemsetAsync(x_dev, 0, d * sizeof(double), st));
    info.it = 0;
    info.flag = 0;
    bool solved = false;
    if (cpqr_on) {
        // explicit sketch solution xs = P1 M c, early exit (:93-117)
        precond_apply(P, cvec, x_dev, ysplit, st);
        residual();
        info.explicit_residual = rnorm;
        solved = rnorm < o.abs_tol;
    }
    SKL_CUDA(cudaEventRecord(ev[5], st));
    if (!solved) {
        // LSQR on A P1 M from r_s (CPQR path) or from b with y = 0 (noCPQR path)
        const double* rhs = b;
        if (cpqr_on) rhs = rs;
        LsqrResult R = lsqr_run(P, rhs, o.it_tol, o.max_it, yv, work, C.dev_status, C.host_pinned,
                                st, o.profile, C.stream);
        add_prof(R);
        int64_t total_it = R.it;
        int flag = R.flag;
        // x = x_s + P1 M y (src/ls_dense_hashing_blendenpik.cpp:130-144; x_s = 0
        // on the noCPQR path): the correction is added to the rounded x_s that
        // r_s was formed from
        SKL_CUDA(cudaMemsetAsync(xacc, 0, d * sizeof(double), st));
        precond_apply(P, yv, xacc, ysplit, st);
        vec_add(x_dev, xacc, d, st);
        residual();
        int64_t restarts = 0;
        while (o.backward_tol > 0.0 && be > o.backward_tol && restarts < o.max_refine &&
               total_it < o.max_it) {
            ++restarts;
            R = lsqr_run(P, rs, o.it_tol, o.max_it - total_it, yv, work, C.dev_status,
                         C.host_pinned, st, o.profile, C.stream);
            add_prof(R);
            total_it += R.it;
            flag = R.flag;
            SKL_CUDA(cudaMemsetAsync(xacc, 0, d * sizeof(double), st));
            precond_apply(P, yv, xacc, ysplit, st);
            vec_add(x_dev, xacc, d, st);
            residual();
        }
        info.it = total_it;
        info.flag = flag;
    }
    SKL_CUDA(cudaEventRecord(ev[6], st));
    SKL_CUDA(cudaEventSynchronize(ev[6]));
    info.residual_norm = rnorm;
    info.backward_error = be;
    info.t_setup_ms = elapsed(ev[1], ev[2]);
    info.t_sketch_ms = elapsed(ev[2], ev[3]);
    info.t_qr_ms = elapsed(ev[3], ev[4]);
    info.t_precond_ms = elapsed(ev[4], ev[5]);
    info.t_lsqr_ms = elapsed(ev[5], ev[6]);
    info.t_total_ms = elapsed(timing_upload ? ev[0] : ev[1], ev[6]);
    if (timing_upload) info.t_upload_ms = elapsed(ev[0], ev[1]);
    return true;
}

// The mixed pipeline, or the FP64 one when the mixed one declines the input.
static void dense_pipeline_any(Context& C, cudaStream_t st, const double* A, int64_t lda,
                               int64_t n, int64_t d, const double* b, double* x_dev,
                               const skl_opts& o, skl_info& info, bool timing_upload,
                               std::thread* host_thread, const std::vector<double>* hD,
                               const std::vector<uint32_t>* hh, int64_t N, bool sample_rows)
{
    if (o.precision == SKL_PREC_MIXED &&
        dense_pipeline<float>(C, st, A, lda, n, d, b, x_dev, o, info, timing_upload, host_thread,
                              hD, hh, N, sample_rows))
        return;
    const bool fell_back = o.precision == SKL_PREC_MIXED;
    if (fell_back) {
        std::memset(&info, 0, sizeof info);
        info.fp64_fallback = 1;
    }
    skl_opts o64 = o;
    o64.precision = SKL_PREC_FP64;
    dense_pipeline<double>(C, st, A, lda, n, d, b, x_dev, o64, info, timing_upload, host_thread,
                           hD, hh, N, sample_rows);
}

static void dense_solve_common(const double* A, int64_t lda, int64_t n, int64_t d, const double* b,
                               double* x, const skl_opts* opts, skl_info* info, bool host,
                               bool sample_rows = false)
{
    skl_opts o;
    if (opts) o = *opts;
    else fill_default(&o);
    if (sample_rows) {
        // Blendenpik: unpivoted QR, no early exit, one "bucket" per sampled row
        o.k = 1;
        o.use_cpqr = 0;
        o.abs_tol = 0.0;
    }
    check_opts(o);
    if (n < 0 || d < 0) fail(SKL_ERR_INVALID, "negative dimension");
    if (n < d) fail(SKL_ERR_NOT_OVERDETERMINED, "Matrix is not overdetermined.");
    if (!A || !b || !x) fail(SKL_ERR_INVALID, "A, b or x is null");
    if (lda < std::max<int64_t>(1, n)) fail(SKL_ERR_INVALID, "lda < n");
    skl_info inf;
    std::memset(&inf, 0, sizeof inf);
    if (d == 0) {
        if (info) *info = inf;
        return;
    }
    Context& C = context(o.device);
    reset_launch_count();
    cudaStream_t st = o.stream ? (cudaStream_t)o.stream : C.stream;
    const int64_t N = dht_length(n, o.wisdom);
    const int64_t m = (int64_t)std::ceil((double)d * o.gamma);
    if (o.k > m) fail(SKL_ERR_INVALID, "k exceeds the sketch size m = ceil(gamma*d)");
    if (N > 0x7fffffff || m > 0x7fffffff) fail(SKL_ERR_INVALID, "problem too large");
    if (sample_rows && m > N)
        fail(SKL_ERR_INVALID, "the sample has more rows (ceil(gamma*d)) than the transform");
    // signs then hash from one reseeded stream (srand(time(NULL)) in the
    // reference, src/dense_helpers.cpp:92 and :12; seed 0 selects time)
    const uint32_t seed = o.seed ? o.seed : (uint32_t)time(nullptr);
    std::vector<double> hD((size_t)n);
    std::vector<uint32_t> hh((size_t)(sample_rows ? m : N * o.k));
    double hash_ms = 0.0;
    const bool hqrrp_stream = o.use_cpqr && std::min(m, d) >= 1000;
    std::thread th([&]() {
        auto t0 = std::chrono::steady_clock::now();
        rng_srand(seed);
        rng_lock();
        gen_signs(n, hD.data());
        if (sample_rows) {
            // random_sample reseeds before its draw (src/dense_helpers.cpp:26)
            rng_unlock();
            rng_srand(seed);
            rng_lock();
            gen_subsample(N, m, hh.data());
        } else {
            gen_hash_packed(m, N, o.k, hh.data());
        }
        rng_unlock();
        hash_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    });
    struct Joiner {
        std::thread& t;
        ~Joiner() { if (t.joinable()) t.join(); }
    } joiner{th};
    SKL_CUDA(cudaEventRecord(C.ev[0], st));
    if (host) {
        Sizer S;
        S.add<double>(n * d); S.add<double>(n); S.add<double>(d);
        C.staging.reserve(S.bytes());
        C.staging.reset();
        double* Ad = C.staging.alloc<double>(n * d);
        double* bd = C.staging.alloc<double>(n);
        double* xd = C.staging.alloc<double>(d);
        if (lda == n)   // one contiguous copy: a pitched copy of d columns runs far below the link rate
            SKL_CUDA(cudaMemcpyAsync(Ad, A, (size_t)n * d * sizeof(double), cudaMemcpyHostToDevice, st));
        else
            SKL_CUDA(cudaMemcpy2DAsync(Ad, n * sizeof(double), A, lda * sizeof(double), n * sizeof(double),
                                       d, cudaMemcpyHostToDevice, st));
        SKL_CUDA(cudaMemcpyAsync(bd, b, n * sizeof(double), cudaMemcpyHostToDevice, st));
        dense_pipeline_any(C, st, Ad, n, n, d, bd, xd, o, inf, true, &th, &hD, &hh, N, sample_rows);
        SKL_CUDA(cudaMemcpyAsync(x, xd, d * sizeof(double), cudaMemcpyDeviceToHost, st));
        SKL_CUDA(cudaStreamSynchronize(st));
    } else {
        dense_pipeline_any(C, st, A, lda, n, d, b, x, o, inf, false, &th, &hD, &hh, N, sample_rows);
    }
    // HQRRP reseeds the C library stream with srand(12) and draws its Gaussian
    // sample (hqrrp/.../NoFLA_HQRRP_WY_blk_var4_skint.c:390,414) when
    // min(m,d) >= 1000; leave the library stream where the reference leaves it.
    if (hqrrp_stream) rng_hqrrp_advance(64 + 10, m);
    inf.t_host_hash_ms = hash_ms;
    inf.kernel_launches = launches_since_reset();
    if (info) *info = inf;
}

}  // namespace skl

using namespace skl;

extern "C" {

void skl_default_opts(skl_opts* opts)
{
    if (opts) fill_default(opts);
}

const char* skl_last_error(void) { return t_last_error.c_str(); }

const char* skl_version(void) { return "skills_gb300 0.1 (sm_103a)"; }

skl_status skl_sparse_solve(const skl_csc* A, const double* b, double* x, const skl_opts* opts,
                            skl_info* info)
{
    return guarded([&] { sparse_solve_common(A, b, x, opts, info, true); });
}

skl_status skl_sparse_solve_device(const skl_csc* A, const double* b, double* x,
                                   const skl_opts* opts, skl_info* info)
{
    return guarded([&] { sparse_solve_common(A, b, x, opts, info, false); });
}

skl_status skl_batched_sparse_solve(int64_t nprob, const skl_csc* A, const double* const* b,
                                    double* const* x, const skl_opts* opts, skl_info* info,
                                    skl_status* status)
{
    return guarded([&] { batched_sparse_common(nprob, A, b, x, opts, info, status); });
}

skl_status skl_dense_solve(const double* A, int64_t lda, int64_t n, int64_t d, const double* b,
                           double* x, const skl_opts* opts, skl_info* info)
{
    return guarded([&] { dense_solve_common(A, lda, n, d, b, x, opts, info, true); });
}

skl_status skl_dense_solve_device(const double* A, int64_t lda, int64_t n, int64_t d,
                                  const double* b, double* x, const skl_opts* opts, skl_info* info)
{
    return guarded([&] { dense_solve_common(A, lda, n, d, b, x, opts, info, false); });
}

skl_status skl_dense_blendenpik_solve(const double* A, int64_t lda, int64_t n, int64_t d,
                                      const double* b, double* x, const skl_opts* opts,
                                      skl_info* info)
{
    return guarded([&] { dense_solve_common(A, lda, n, d, b, x, opts, info, true, true); });
}

skl_status skl_dense_blendenpik_solve_device(const double* A, int64_t lda, int64_t n, int64_t d,
                                             const double* b, double* x, const skl_opts* opts,
                                             skl_info* info)
{
    return guarded([&] { dense_solve_common(A, lda, n, d, b, x, opts, info, false, true); });
}

void skl_finalize(void)
{
    release_all_contexts();
    noalloc_forget_scratch();
    tune_cache_clear();
}

}  // extern "C"
