// skl_blocks.cpp -- building-block entry points of the C ABI: each runs one
// stage of the GPU solve path on host data, so the stage can be checked in
// isolation against the reference's function of the same role.
#include <cmath>
#include <cstring>
#include <algorithm>
#include <functional>
#include <type_traits>
#include <vector>

#include "skl_internal.hpp"

namespace skl {

static skl_status guard(const std::function<void()>& f)
{
    struct Box { const std::function<void()>* f; } box{&f};
    return run_guarded([](void* a) { (*((Box*)a)->f)(); }, &box);
}

template <typename T>
static void to_device_as(const double* h, int64_t rows, int64_t cols, int64_t ldh, T* d,
                         int64_t ldd, cudaStream_t st)
{
    std::vector<T> tmp((size_t)(ldd * cols), T(0));
    for (int64_t j = 0; j < cols; ++j)
        for (int64_t i = 0; i < rows; ++i) tmp[(size_t)(i + j * ldd)] = (T)h[i + j * ldh];
    SKL_CUDA(cudaMemcpyAsync(d, tmp.data(), tmp.size() * sizeof(T), cudaMemcpyHostToDevice, st));
    SKL_CUDA(cudaStreamSynchronize(st));
}

template <typename T>
static void from_device_as(const T* d, int64_t rows, int64_t cols, int64_t ldd, double* h,
                           int64_t ldh, cudaStream_t st)
{
    std::vector<T> tmp((size_t)(ldd * cols));
    SKL_CUDA(cudaMemcpyAsync(tmp.data(), d, tmp.size() * sizeof(T), cudaMemcpyDeviceToHost, st));
    SKL_CUDA(cudaStreamSynchronize(st));
    for (int64_t j = 0; j < cols; ++j)
        for (int64_t i = 0; i < rows; ++i) h[i + j * ldh] = (double)tmp[(size_t)(i + j * ldd)];
}

template <typename T>
static void sketch_sparse_block(const skl_csc* A, const double* b, int64_t m, int64_t k,
                                const int64_t* rows, const double* vals, int equilibrate,
                                double* SA, double* Sb)
{
    Context& C = context(0);
    cudaStream_t st = C.stream;
    const int64_t n = A->m, d = A->n, nnz = A->p[d];
    Sizer S;
    S.add<int64_t>(d + 1); S.add<int64_t>(nnz); S.add<double>(nnz); S.add<double>(n);
    S.add<int>(d + 1); S.add<int>(nnz); S.add<unsigned>(n * k); S.add<int>(m + 1);
    S.add<unsigned>(n * k); S.add<T>(m * d); S.add<double>(d); S.add<double>(d); S.add<double>(m);
    S.add<int>((int64_t)build_buckets_scratch_ints(m, n * k));
    C.arena.reserve(S.bytes());
    C.arena.reset();
    Arena& Ar = C.arena;
    int64_t* Ap = Ar.alloc<int64_t>(d + 1);
    int64_t* Ai = Ar.alloc<int64_t>(nnz);
    double* Ax = Ar.alloc<double>(nnz);
    double* bd = Ar.alloc<double>(n);
    int* cp = Ar.alloc<int>(d + 1);
    int* ri = Ar.alloc<int>(nnz);
    unsigned* hidx = Ar.alloc<unsigned>(n * k);
    int* bptr = Ar.alloc<int>(m + 1);
    unsigned* bent = Ar.alloc<unsigned>(n * k);
    T* SAd = Ar.alloc<T>(m * d);
    double* cn = Ar.alloc<double>(d);
    double* cs = Ar.alloc<double>(d);
    double* Sbd = Ar.alloc<double>(m);
    int* scr = Ar.alloc<int>((int64_t)build_buckets_scratch_ints(m, n * k));
    std::vector<uint32_t> h((size_t)(n * k));
    for (int64_t q = 0; q < n * k; ++q) {
        if (rows[q] < 0 || rows[q] >= m) fail(SKL_ERR_INVALID, "hash row out of range");
        h[(size_t)q] = (uint32_t)rows[q] | (vals[q] < 0 ? 0x80000000u : 0u);
    }
    SKL_CUDA(cudaMemcpyAsync(Ap, A->p, (d + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    if (nnz) {
        SKL_CUDA(cudaMemcpyAsync(Ai, A->i, nnz * sizeof(int64_t), cudaMemcpyHostToDevice, st));
        SKL_CUDA(cudaMemcpyAsync(Ax, A->x, nnz * sizeof(double), cudaMemcpyHostToDevice, st));
    }
    SKL_CUDA(cudaMemcpyAsync(bd, b, n * sizeof(double), cudaMemcpyHostToDevice, st));
    SKL_CUDA(cudaMemcpyAsync(hidx, h.data(), n * k * sizeof(unsigned), cudaMemcpyHostToDevice, st));
    SKL_CUDA(cudaMemsetAsync(C.dev_status, 0, sizeof(unsigned), st));
    csc_narrow(Ap, Ai, Ax, n, d, nnz, cp, ri, C.dev_status, st);
    build_buckets(hidx, n, (int)k, m, bptr, bent, scr, st);
    sketch_sparse<T>(cp, ri, Ax, n, d, hidx, (int)k, m, SAd, m, equilibrate, cn, cs, st);
    sketch_rhs(bptr, bent, m, (int)k, bd, Sbd, st);
    from_device_as<T>(SAd, m, d, m, SA, m, st);
    SKL_CUDA(cudaMemcpyAsync(Sb, Sbd, m * sizeof(double), cudaMemcpyDeviceToHost, st));
    SKL_CUDA(cudaStreamSynchronize(st));
}

template <typename T>
static void cpqr_block(double* A, int64_t m, int64_t d, int64_t* jpvt, double* tau)
{
    Context& C = context(0);
    cudaStream_t st = C.stream;
    const int64_t ld = (m + 31) / 32 * 32, mn = m < d ? m : d;
    const size_t ws = cpqr_workspace_bytes<T>(m, d);
    Sizer S;
    S.add<T>(ld * d); S.add<int>(d); S.add<T>(mn); S.add<char>((int64_t)ws);
    C.arena.reserve(S.bytes());
    C.arena.reset();
    T* Ad = C.arena.alloc<T>(ld * d);
    int* jp = C.arena.alloc<int>(d);
    T* td = C.arena.alloc<T>(mn);
    void* work = C.arena.take(ws);
    to_device_as<T>(A, m, d, m, Ad, ld, st);
    SKL_CUDA(cudaMemsetAsync(C.dev_status, 0, sizeof(unsigned), st));
    cpqr<T>(Ad, m, d, ld, jp, td, work, C.dev_status, st, nullptr, 1);
    {
        unsigned stt = 0;
        SKL_CUDA(cudaMemcpyAsync(&stt, C.dev_status, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        SKL_CUDA(cudaStreamSynchronize(st));
        if (stt & kStatusTcTimeout) fail(SKL_ERR_TIMEOUT, "a tensor-core kernel's bounded wait gave up");
        if (stt & 8u) fail(SKL_ERR_NONFINITE, "non-finite values in the sketch factorization");
    }
    from_device_as<T>(Ad, m, d, ld, A, m, st);
    std::vector<int> hj((size_t)d);
    std::vector<T> ht((size_t)mn);
    SKL_CUDA(cudaMemcpyAsync(hj.data(), jp, d * sizeof(int), cudaMemcpyDeviceToHost, st));
    SKL_CUDA(cudaMemcpyAsync(ht.data(), td, mn * sizeof(T), cudaMemcpyDeviceToHost, st));
    SKL_CUDA(cudaStreamSynchronize(st));
    for (int64_t j = 0; j < d; ++j) jpvt[j] = hj[(size_t)j];
    for (int64_t j = 0; j < mn; ++j) tau[j] = (double)ht[(size_t)j];
}

template <typename T>
static void trsv_block(const double* R, int64_t ld, int64_t r, char trans, double* x)
{
    Context& C = context(0);
    cudaStream_t st = C.stream;
    const size_t ws = trinv_workspace_bytes<T>(r);
    Sizer S;
    S.add<T>(r * r); S.add<T>(r * r); S.add<double>(4); S.add<double>(r); S.add<double>(r);
    S.add<char>((int64_t)ws);
    C.arena.reserve(S.bytes());
    C.arena.reset();
    T* Rd = C.arena.alloc<T>(r * r);
    T* Md = C.arena.alloc<T>(r * r);
    double* norms = C.arena.alloc<double>(4);
    double* xd = C.arena.alloc<double>(r);
    double* yd = C.arena.alloc<double>(r);
    void* work = C.arena.take(ws);
    to_device_as<T>(R, r, r, ld, Rd, r, st);
    SKL_CUDA(cudaMemcpyAsync(xd, x, r * sizeof(double), cudaMemcpyHostToDevice, st));
    trinv_upper<T>(Rd, r, r, 0.0, Md, r, norms, work, st);
    trmv_upper<T>(Md, r, r, (trans == 't' || trans == 'T') ? 1 : 0, xd, yd, st);
    SKL_CUDA(cudaMemcpyAsync(x, yd, r * sizeof(double), cudaMemcpyDeviceToHost, st));
    SKL_CUDA(cudaStreamSynchronize(st));
}

template <typename T>
static void dht_block(const double* A, int64_t lda, int64_t n, int64_t d, const double* D,
                      int64_t N, double* Y)
{
    Context& C = context(0);
    cudaStream_t st = C.stream;
    const size_t scr = dht_scratch_bytes(N, std::is_same<T, float>::value ? SKL_PREC_MIXED : SKL_PREC_FP64);
    Sizer S;
    S.add<double>(n * d); S.add<double>(n); S.add<double>(N * d); S.add<char>((int64_t)scr);
    C.arena.reserve(S.bytes());
    C.arena.reset();
    double* Ad = C.arena.alloc<double>(n * d);
    double* Dd = C.arena.alloc<double>(n);
    double* Yd = C.arena.alloc<double>(N * d);
    void* work = C.arena.take(scr);
    SKL_CUDA(cudaMemcpy2DAsync(Ad, n * sizeof(double), A, lda * sizeof(double), n * sizeof(double), d,
                               cudaMemcpyHostToDevice, st));
    SKL_CUDA(cudaMemcpyAsync(Dd, D, n * sizeof(double), cudaMemcpyHostToDevice, st));
    dht_hash<T>(Ad, n, n, d, Dd, N, nullptr, nullptr, 1, 0, (T*)nullptr, 0, Yd, N, work, scr, st);
    SKL_CUDA(cudaMemcpyAsync(Y, Yd, N * d * sizeof(double), cudaMemcpyDeviceToHost, st));
    SKL_CUDA(cudaStreamSynchronize(st));
}

template <typename T>
static void sketch_dense_block(const double* A, int64_t lda, int64_t n, int64_t d, const double* b,
                               const double* D, int64_t N, int64_t m, int64_t k,
                               const int64_t* rows, const double* vals, double* SA, double* Sb)
{
    Context& C = context(0);
    cudaStream_t st = C.stream;
    const size_t scr = std::max(dht_scratch_bytes(N, SKL_PREC_FP64),
                                build_buckets_scratch_ints(m, N * k) * sizeof(int));
    Sizer S;
    S.add<double>(n * d); S.add<double>(n); S.add<double>(n); S.add<unsigned>(N * k);
    S.add<int>(m + 1); S.add<unsigned>(N * k); S.add<T>(m * d); S.add<double>(m);
    S.add<char>((int64_t)scr);
    C.arena.reserve(S.bytes());
    C.arena.reset();
    double* Ad = C.arena.alloc<double>(n * d);
    double* bd = C.arena.alloc<double>(n);
    double* Dd = C.arena.alloc<double>(n);
    unsigned* hidx = C.arena.alloc<unsigned>(N * k);
    int* bptr = C.arena.alloc<int>(m + 1);
    unsigned* bent = C.arena.alloc<unsigned>(N * k);
    T* SAd = C.arena.alloc<T>(m * d);
    double* Sbd = C.arena.alloc<double>(m);
    void* work = C.arena.take(scr);
    std::vector<uint32_t> h((size_t)(N * k));
    for (int64_t q = 0; q < N * k; ++q) {
        if (rows[q] < 0 || rows[q] >= m) fail(SKL_ERR_INVALID, "hash row out of range");
        h[(size_t)q] = (uint32_t)rows[q] | (vals[q] < 0 ? 0x80000000u : 0u);
    }
    SKL_CUDA(cudaMemcpy2DAsync(Ad, n * sizeof(double), A, lda * sizeof(double), n * sizeof(double), d,
                               cudaMemcpyHostToDevice, st));
    SKL_CUDA(cudaMemcpyAsync(bd, b, n * sizeof(double), cudaMemcpyHostToDevice, st));
    SKL_CUDA(cudaMemcpyAsync(Dd, D, n * sizeof(double), cudaMemcpyHostToDevice, st));
    SKL_CUDA(cudaMemcpyAsync(hidx, h.data(), N * k * sizeof(unsigned), cudaMemcpyHostToDevice, st));
    build_buckets(hidx, N, (int)k, m, bptr, bent, (int*)work, st);
    dht_hash<T>(Ad, n, n, d, Dd, N, bptr, bent, (int)k, m, SAd, m, nullptr, 0, work, scr, st);
    dht_hash_rhs(bd, n, Dd, N, bptr, bent, (int)k, m, Sbd, work, scr, st);
    from_device_as<T>(SAd, m, d, m, SA, m, st);
    SKL_CUDA(cudaMemcpyAsync(Sb, Sbd, m * sizeof(double), cudaMemcpyDeviceToHost, st));
    SKL_CUDA(cudaStreamSynchronize(st));
}

// y = A x or A^T x through LSQR's product kernels.  The mixed path stores the
// equilibrated values A(:, c) / ||A(:, c)|| as (hi, lo) float pairs, as the
// sparse solve does.
static void csc_mv_block(const skl_csc* A, char trans, const double* x, double* y, int precision)
{
    Context& C = context(0);
    cudaStream_t st = C.stream;
    const bool mixed = precision != SKL_PREC_FP64;
    const int64_t n = A->m, d = A->n, nnz = A->p[d];
    if (n > 0x7fffffff || d > 0x7fffffff || nnz > 0x7fffffff)
        fail(SKL_ERR_INVALID, "skl_csc_mv: problem too large for 32-bit device indices");
    std::vector<double> cs((size_t)d, 1.0);
    for (int64_t j = 0; j < d; ++j) {
        double ss = 0.0;
        for (int64_t p = A->p[j]; p < A->p[j + 1]; ++p) ss += A->x[p] * A->x[p];
        if (mixed && ss > 0.0) cs[(size_t)j] = 1.0 / std::sqrt(ss);
    }
    std::vector<int> cols((size_t)d);
    for (int64_t j = 0; j < d; ++j) cols[(size_t)j] = (int)j;
    LsqrProblem P;
    P.n = n; P.d = d; P.nnz = nnz; P.r = d; P.precision = mixed ? SKL_PREC_MIXED : SKL_PREC_FP64;
    const size_t ws = lsqr_workspace_bytes(P);
    Sizer S;
    S.add<int64_t>(d + 1); S.add<int64_t>(nnz); S.add<double>(nnz);
    S.add<int>(d + 1); S.add<int>(nnz); S.add<int>(n + 1); S.add<int>(nnz); S.add<double>(nnz);
    S.add<float2>(nnz); S.add<float2>(nnz); S.add<double>(d); S.add<int>(d);
    S.add<double>(n); S.add<double>(n);
    S.add<char>((int64_t)std::max(ws, build_csr_scratch_ints(n, nnz) * sizeof(int)));
    C.arena.reserve(S.bytes());
    C.arena.reset();
    Arena& Ar = C.arena;
    int64_t* Ap = Ar.alloc<int64_t>(d + 1);
    int64_t* Ai = Ar.alloc<int64_t>(nnz);
    double* Ax = Ar.alloc<double>(nnz);
    int* cp = Ar.alloc<int>(d + 1);
    int* ri = Ar.alloc<int>(nnz);
    int* rp = Ar.alloc<int>(n + 1);
    int* ci = Ar.alloc<int>(nnz);
    double* cx = Ar.alloc<double>(nnz);
    float2* cx2 = Ar.alloc<float2>(nnz);
    float2* rx2 = Ar.alloc<float2>(nnz);
    double* csd = Ar.alloc<double>(d);
    int* colsd = Ar.alloc<int>(d);
    double* xd = Ar.alloc<double>(n);
    double* yd = Ar.alloc<double>(n);
    void* work = Ar.take(std::max(ws, build_csr_scratch_ints(n, nnz) * sizeof(int)));
    SKL_CUDA(cudaMemcpyAsync(Ap, A->p, (d + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    if (nnz) {
        SKL_CUDA(cudaMemcpyAsync(Ai, A->i, nnz * sizeof(int64_t), cudaMemcpyHostToDevice, st));
        SKL_CUDA(cudaMemcpyAsync(Ax, A->x, nnz * sizeof(double), cudaMemcpyHostToDevice, st));
    }
    SKL_CUDA(cudaMemcpyAsync(csd, cs.data(), d * sizeof(double), cudaMemcpyHostToDevice, st));
    SKL_CUDA(cudaMemcpyAsync(colsd, cols.data(), d * sizeof(int), cudaMemcpyHostToDevice, st));
    const int64_t lin = trans == 'n' ? d : n, lout = trans == 'n' ? n : d;
    SKL_CUDA(cudaMemcpyAsync(xd, x, lin * sizeof(double), cudaMemcpyHostToDevice, st));
    SKL_CUDA(cudaMemsetAsync(C.dev_status, 0, sizeof(unsigned), st));
    csc_narrow(Ap, Ai, Ax, n, d, nnz, cp, ri, C.dev_status, st);
    build_csr(cp, ri, Ax, n, d, nnz, rp, ci, cx, (int*)work, st);
    {
        unsigned stt = 0;
        SKL_CUDA(cudaMemcpyAsync(&stt, C.dev_status, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        SKL_CUDA(cudaStreamSynchronize(st));
        if (stt & 3u) fail(SKL_ERR_INVALID, "skl_csc_mv: invalid CSC structure");
        if (stt & 4u) fail(SKL_ERR_NONFINITE, "A contains NaN or Inf");
    }
    if (mixed) {
        split_csr_scaled(ci, cx, nnz, csd, cx2, st);
        split_csc_scaled(cp, Ax, d, csd, rx2, st);
    }
    P.rp = rp; P.ci = ci; P.cx = mixed ? (const void*)cx2 : (const void*)cx;
    P.cp = cp; P.ri = ri; P.rx = mixed ? (const void*)rx2 : (const void*)Ax;
    P.cols = colsd; P.colscale = csd; P.opscale = nullptr;
    lsqr_product(P, trans, xd, yd, mixed ? csd : nullptr, work, st);
    SKL_CUDA(cudaMemcpyAsync(y, yd, lout * sizeof(double), cudaMemcpyDeviceToHost, st));
    SKL_CUDA(cudaStreamSynchronize(st));
}

// W = V^T A (FP32) through the CPQR's product for the block reflector:
// tensor = 1 the tcgen05 3xTF32 kernel, 0 the CUDA-core FP32 kernel.
static void gemm_vta_block(int64_t M, int64_t N, int64_t b, const float* V, int64_t ldv,
                           const float* A, int64_t lda, float* W, int tensor)
{
    Context& C = context(0);
    cudaStream_t st = C.stream;
    const int64_t ldd = (M + 31) / 32 * 32;
    const size_t scr = std::max(tc_vta_scratch_floats(M), (size_t)(b * N * 128));
    Sizer S;
    S.add<float>(ldd * b); S.add<float>(ldd * N); S.add<float>(b * N); S.add<float>((int64_t)scr);
    C.arena.reserve(S.bytes());
    C.arena.reset();
    float* Vd = C.arena.alloc<float>(ldd * b);
    float* Ad = C.arena.alloc<float>(ldd * N);
    float* Wd = C.arena.alloc<float>(b * N);
    float* sd = C.arena.alloc<float>((int64_t)scr);
    SKL_CUDA(cudaMemcpy2DAsync(Vd, ldd * sizeof(float), V, ldv * sizeof(float), M * sizeof(float), b,
                               cudaMemcpyHostToDevice, st));
    SKL_CUDA(cudaMemcpy2DAsync(Ad, ldd * sizeof(float), A, lda * sizeof(float), M * sizeof(float), N,
                               cudaMemcpyHostToDevice, st));
    SKL_CUDA(cudaMemsetAsync(C.dev_status, 0, sizeof(unsigned), st));
    vta_product(tensor != 0, (int)M, (int)N, (int)b, Vd, ldd, Ad, ldd, Wd, sd, scr, C.dev_status, st);
    unsigned stt = 0;
    SKL_CUDA(cudaMemcpyAsync(&stt, C.dev_status, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    SKL_CUDA(cudaMemcpyAsync(W, Wd, b * N * sizeof(float), cudaMemcpyDeviceToHost, st));
    SKL_CUDA(cudaStreamSynchronize(st));
    if (stt & kStatusTcTimeout) fail(SKL_ERR_TIMEOUT, "a tensor-core kernel's bounded wait gave up");
}

// C (M x N) rows r0.. -= V Z (FP32): the trailing update of the CPQR.
static void gemm_update_block(int64_t M, int64_t N, int64_t b, int64_t r0, const float* V, int64_t ldv,
                              const float* Z, int64_t ldz, float* C, int64_t ldc, int tensor)
{
    Context& Cx = context(0);
    cudaStream_t st = Cx.stream;
    const int64_t ldd = (M + 31) / 32 * 32;
    const size_t scr = tc_update_scratch_floats(M, N);
    Sizer S;
    S.add<float>(ldd * b); S.add<float>(b * N); S.add<float>(ldd * N); S.add<float>((int64_t)scr);
    Cx.arena.reserve(S.bytes());
    Cx.arena.reset();
    float* Vd = Cx.arena.alloc<float>(ldd * b);
    float* Zd = Cx.arena.alloc<float>(b * N);
    float* Cd = Cx.arena.alloc<float>(ldd * N);
    float* sd = Cx.arena.alloc<float>((int64_t)scr);
    SKL_CUDA(cudaMemcpy2DAsync(Vd, ldd * sizeof(float), V, ldv * sizeof(float), M * sizeof(float), b,
                               cudaMemcpyHostToDevice, st));
    SKL_CUDA(cudaMemcpy2DAsync(Zd, b * sizeof(float), Z, ldz * sizeof(float), b * sizeof(float), N,
                               cudaMemcpyHostToDevice, st));
    SKL_CUDA(cudaMemcpy2DAsync(Cd, ldd * sizeof(float), C, ldc * sizeof(float), M * sizeof(float), N,
                               cudaMemcpyHostToDevice, st));
    SKL_CUDA(cudaMemsetAsync(Cx.dev_status, 0, sizeof(unsigned), st));
    update_product(tensor != 0, (int)M, (int)N, (int)b, (int)r0, Vd, ldd, Zd, b, Cd, ldd, sd,
                   Cx.dev_status, st);
    unsigned stt = 0;
    SKL_CUDA(cudaMemcpyAsync(&stt, Cx.dev_status, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    SKL_CUDA(cudaMemcpy2DAsync(C, ldc * sizeof(float), Cd, ldd * sizeof(float), M * sizeof(float), N,
                               cudaMemcpyDeviceToHost, st));
    SKL_CUDA(cudaStreamSynchronize(st));
    if (stt & kStatusTcTimeout) fail(SKL_ERR_TIMEOUT, "a tensor-core kernel's bounded wait gave up");
}

}  // namespace skl

using namespace skl;

extern "C" {

skl_status skl_sketch_sparse(const skl_csc* A, const double* b, int64_t m, int64_t k,
                             const int64_t* rows, const double* vals, int precision,
                             int equilibrate, double* SA, double* Sb)
{
    return guard([&] {
        if (!A || !A->p || !b || !rows || !vals || !SA || !Sb || m <= 0 || k < 1)
            fail(SKL_ERR_INVALID, "skl_sketch_sparse: bad argument");
        if (precision == SKL_PREC_FP64)
            sketch_sparse_block<double>(A, b, m, k, rows, vals, equilibrate, SA, Sb);
        else
            sketch_sparse_block<float>(A, b, m, k, rows, vals, equilibrate, SA, Sb);
    });
}

skl_status skl_cpqr(double* A, int64_t m, int64_t d, int precision, int64_t* jpvt, double* tau)
{
    return guard([&] {
        if (!A || !jpvt || !tau || m <= 0 || d <= 0) fail(SKL_ERR_INVALID, "skl_cpqr: bad argument");
        if (precision == SKL_PREC_FP64) cpqr_block<double>(A, m, d, jpvt, tau);
        else cpqr_block<float>(A, m, d, jpvt, tau);
    });
}

skl_status skl_trsv_upper(const double* R, int64_t ld, int64_t r, char trans, int precision,
                          double* x)
{
    return guard([&] {
        if (!R || !x || r <= 0 || ld < r) fail(SKL_ERR_INVALID, "skl_trsv_upper: bad argument");
        if (precision == SKL_PREC_FP64) trsv_block<double>(R, ld, r, trans, x);
        else trsv_block<float>(R, ld, r, trans, x);
    });
}

skl_status skl_gemm_vta(int64_t M, int64_t N, int64_t b, const float* V, int64_t ldv,
                        const float* A, int64_t lda, float* W, int tensor)
{
    return guard([&] {
        if (!V || !A || !W || M <= 0 || N <= 0 || b <= 0 || b > 64 || ldv < M || lda < M ||
            M > 0x7fffffff || N > 0x7fffffff)
            fail(SKL_ERR_INVALID, "skl_gemm_vta: bad argument");
        gemm_vta_block(M, N, b, V, ldv, A, lda, W, tensor);
    });
}

skl_status skl_gemm_update(int64_t M, int64_t N, int64_t b, int64_t r0, const float* V, int64_t ldv,
                           const float* Z, int64_t ldz, float* C, int64_t ldc, int tensor)
{
    return guard([&] {
        if (!V || !Z || !C || M <= 0 || N <= 0 || b <= 0 || b > 64 || r0 < 0 || r0 > M || (r0 & 3) ||
            ldv < M || ldz < b || ldc < M || M > 0x7fffffff || N > 0x7fffffff)
            fail(SKL_ERR_INVALID, "skl_gemm_update: bad argument");
        gemm_update_block(M, N, b, r0, V, ldv, Z, ldz, C, ldc, tensor);
    });
}

skl_status skl_csc_mv(const skl_csc* A, char trans, const double* x, double* y, int precision)
{
    return guard([&] {
        if (!A || !A->p || !x || !y || A->m < 0 || A->n < 0 || (trans != 'n' && trans != 't'))
            fail(SKL_ERR_INVALID, "skl_csc_mv: bad argument");
        if (A->p[A->n] > 0 && (!A->i || !A->x)) fail(SKL_ERR_INVALID, "skl_csc_mv: bad argument");
        if (A->m == 0 || A->n == 0) {
            const int64_t lout = trans == 'n' ? A->m : A->n;
            for (int64_t i = 0; i < lout; ++i) y[i] = 0.0;
            return;
        }
        csc_mv_block(A, trans, x, y, precision);
    });
}

skl_status skl_dht(const double* A, int64_t lda, int64_t n, int64_t d, const double* D, int64_t N,
                   int precision, double* Y)
{
    return guard([&] {
        if (!A || !D || !Y || n <= 0 || d <= 0 || lda < n || N < n)
            fail(SKL_ERR_INVALID, "skl_dht: bad argument");
        if (precision == SKL_PREC_FP64) dht_block<double>(A, lda, n, d, D, N, Y);
        else dht_block<float>(A, lda, n, d, D, N, Y);
    });
}

int64_t skl_dht_length(int64_t n, int wisdom) { return dht_length(n, wisdom); }

skl_status skl_sketch_dense(const double* A, int64_t lda, int64_t n, int64_t d, const double* b,
                            const double* D, int64_t N, int64_t m, int64_t k, const int64_t* rows,
                            const double* vals, int precision, double* SA, double* Sb)
{
    return guard([&] {
        if (!A || !b || !D || !rows || !vals || !SA || !Sb || n <= 0 || d <= 0 || lda < n ||
            N < n || m <= 0 || k < 1)
            fail(SKL_ERR_INVALID, "skl_sketch_dense: bad argument");
        if (precision == SKL_PREC_FP64)
            sketch_dense_block<double>(A, lda, n, d, b, D, N, m, k, rows, vals, SA, Sb);
        else
            sketch_dense_block<float>(A, lda, n, d, b, D, N, m, k, rows, vals, SA, Sb);
    });
}

}  // extern "C"
