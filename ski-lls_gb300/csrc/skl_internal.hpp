// skl_internal.hpp -- host-side internals shared by the solver's translation units.
#pragma once
#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>

#include <cuda_runtime.h>

#include "../../include/skills_gb300.h"

namespace skl {

// Internal failures travel as exceptions and are turned into skl_status at
// the C ABI (no exception crosses the boundary).
struct Error : std::runtime_error {
    skl_status status;
    Error(skl_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

[[noreturn]] void fail(skl_status s, const std::string& msg);
void check_cuda(cudaError_t e, const char* what, const char* file, int line);
#define SKL_CUDA(x) ::skl::check_cuda((x), #x, __FILE__, __LINE__)

// Phase tracing (SKILLS_TRACE=1): synchronises the stream after each phase and
// prints the phase name and the elapsed host time to stderr.
void trace_phase(cudaStream_t st, const char* name);

// Raise a kernel's dynamic shared-memory limit to the device maximum (less
// its static shared memory).  Always the same value, so concurrent solves on
// several host threads can call it before any launch without lowering the
// limit under one another.
void allow_max_dynamic_smem(const void* fn);

// Kernel launch accounting (counted per solve, reported in skl_info).
void note_launch();
int64_t launches_since_reset();
void reset_launch_count();
#define SKL_LAUNCHED() ::skl::note_launch()

// Grow-only device arena; one per device context, bump-allocated per solve.
class Arena {
public:
    void reserve(size_t bytes);
    void reset() { used_ = 0; }
    void* take(size_t bytes);
    template <typename T>
    T* alloc(int64_t count) { return static_cast<T*>(take((size_t)(count > 0 ? count : 1) * sizeof(T))); }
    size_t capacity() const { return cap_; }
    size_t used() const { return used_; }
    void release();
    ~Arena() { release(); }

private:
    char* base_ = nullptr;
    size_t cap_ = 0, used_ = 0;
};

// Computes the arena size of a sequence of allocations before reserving it.
class Sizer {
public:
    template <typename T>
    void add(int64_t count) { bytes_ += ((size_t)(count > 0 ? count : 1) * sizeof(T) + 255) & ~(size_t)255; }
    size_t bytes() const { return bytes_ + 4096; }

private:
    size_t bytes_ = 0;
};

struct Context {
    int device = -1;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[16] = {};
    Arena arena;
    Arena staging;           // device copies of host inputs
    unsigned* dev_status = nullptr;  // device error word (kDevErr*)
    double* dev_scalars = nullptr;   // small pinned-size scalar area (device)
    void* host_pinned = nullptr;     // pinned host scratch for scalar readback
    size_t host_pinned_bytes = 0;
};

// Device context `slot` of a device (slot 0: single solves; 1..: batched workers).
Context& context(int device, int slot = 0);
// Runs fn and converts exceptions into an skl_status (C ABI guard).
skl_status run_guarded(void (*fn)(void*), void* arg);
void release_all_contexts();
// Forgets skl_dht_device_noalloc's per-device scratch addresses (k_noalloc.cu).
void noalloc_forget_scratch();
// Clears the autotuner's per-shape-class launch choices.
void tune_cache_clear();

// ---------------------------------------------------------- k_format.cu --
size_t scan_scratch_ints(int64_t n);
void scan_exclusive(const int* in, int64_t n, int* out, int* scratch, cudaStream_t st);
size_t radix_sort_scratch_ints(int64_t n);
void radix_sort_pairs(unsigned* keys, unsigned* vals, unsigned* keys_tmp, unsigned* vals_tmp,
                      int64_t n, int bits, int* scratch, cudaStream_t st);
int bits_for(int64_t maxval);
void csc_narrow(const int64_t* Ap, const int64_t* Ai, const double* Ax, int64_t nrow, int64_t ncol,
                int64_t nnz, int* cp, int* ri, unsigned* bad, cudaStream_t st);
size_t build_csr_scratch_ints(int64_t nrow, int64_t nnz);
void build_csr(const int* cp, const int* ri, const double* Ax, int64_t nrow, int64_t ncol,
               int64_t nnz, int* rp, int* ci, double* cx, int* scratch, cudaStream_t st);
// Flags bit 16 of *status if a hashed row index is outside [0, m).
void check_hash_rows(const unsigned* hidx, int64_t nk, int64_t m, unsigned* status, cudaStream_t st);
size_t build_buckets_scratch_ints(int64_t m, int64_t nk);
void build_buckets(const unsigned* hidx, int64_t n, int k, int64_t m, int* bptr, unsigned* bent,
                   int* scratch, cudaStream_t st);

// ---------------------------------------------------------- k_sketch.cu --
// Sparse sketch: SA (m x d, ld) = S*A with column j scaled by colscale[j]
// (written by the kernel: 1/||A(:,j)|| if equilibrate else 1); Sb = S*b.
// threads: block size of the one-CTA-per-column kernel (256, 512 or 1024;
// 0 = 512), a tuning choice (S A itself is exact fixed point; the column
// norms' summation order follows the block size).
template <typename T>
void sketch_sparse(const int* cp, const int* ri, const double* Ax, int64_t n, int64_t d,
                   const unsigned* hidx, int k, int64_t m, T* SA, int64_t ld, int equilibrate,
                   double* colnorm, double* colscale, cudaStream_t st, int threads = 0);
void sketch_rhs(const int* bptr, const unsigned* bent, int64_t m, int k, const double* b,
                double* Sb, cudaStream_t st);
// ----------------------------------------------------------- k_dense.cu --
// Dense path: Y = DHT_N(D*A/sqrt(N)) column by column (n x d, lda; zero padded
// to N), hashed into SA (m x d, ld) through S's buckets with the net factor
// (1/sqrt(k))^2; optionally Y itself to Yout (N x d, ldy).  FP64 columns use
// `scratch` (dht_scratch_bytes).
int64_t dht_length(int64_t n, int wisdom);
size_t dht_scratch_bytes(int64_t N, int precision);
// Load the DHT kernels' module on the current device (one-time set-up).
void dht_load_kernels();

// ---------------------------------------------------------- k_qr_chol.cu --
// CholeskyQR2 + Householder reconstruction of one QR panel P (M x b) =
// A(j0:, j0:j0+b) (FP32 only): V, T, tau and the panel of A on success;
// *fail = 1 and A untouched otherwise.  cg, cr1, cx1, cw: b x b scratch;
// tmp: M x b; part: split-K partials.
template <typename T>
void chol_panel(T* P, int64_t ld, int M, int b, int j0, T* A, T* cg, T* cr1, T* cx1, T* cw, T* tmp,
                T* V, int64_t ldv, T* Tm, int ldt, T* tau, T* part, int64_t part_cap, int* fail,
                cudaStream_t st);
template <typename T>
void dht_hash(const double* A, int64_t lda, int64_t n, int64_t d, const double* D, int64_t N,
              const int* bptr, const unsigned* bent, int k, int64_t m, T* SA, int64_t ld,
              double* Yout, int64_t ldy, void* scratch, size_t scratch_bytes, cudaStream_t st);
void dht_hash_rhs(const double* b, int64_t n, const double* D, int64_t N, const int* bptr,
                  const unsigned* bent, int k, int64_t m, double* Sb, void* scratch,
                  size_t scratch_bytes, cudaStream_t st);
void fro_partials(const double* A, int64_t lda, int64_t n, int64_t d, double* out512,
                  cudaStream_t st);

// -------------------------------------------------------------- k_qr.cu --
template <typename T>
size_t cpqr_workspace_bytes(int64_t m, int64_t d);
// Randomized CPQR in place on A (m x d, ld); jpvt (int, d) receives the
// 0-based column permutation, tau (min(m,d)).  If c != nullptr, c (m
// entries, FP64) is overwritten with Q^T c.  pivoting = 0 gives an unpivoted
// blocked Householder QR (the _noCPQR path).
// qr_prof (optional, host array of kQrProfSlots): summed CUDA-event ms of the
// QR sub-steps: 0 sample QRP, 1 column moves, 2 panel, 3 Q^T c, 4 W = V^T A,
// 5 Z = T^T W, 6 A -= V Z, 7 Y/G downdate, 8 initial sample Y = G A.
constexpr int kQrProfSlots = 9;
// nb_cap > 0 caps the panel width (a multiple of 8; the workspace of the
// default plan covers every smaller width).
template <typename T>
void cpqr(T* A, int64_t m, int64_t d, int64_t ld, int* jpvt, T* tau, void* work,
          unsigned* status, cudaStream_t st, double* c, int pivoting, double* qr_prof = nullptr,
          int nb_cap = 0);
// Panel width the FP32 CPQR uses for m x d under the cap.
int cpqr_panel_width(int64_t m, int64_t d, int nb_cap);

// --------------------------------------------------------------- k_tc.cu --
// Status bit of a kernel whose bounded mbarrier wait gave up (the tensor-core
// products, the sample QRP's candidate exchange).
constexpr unsigned kStatusTcTimeout = 64u;
// W (b x N, ld b) = V^T A on the tensor cores (tcgen05, 3xTF32): V is M x b
// (ldv, b <= 64), A is M x N (lda); both 16-byte aligned with ld*4 a multiple
// of 16 bytes.  scratch holds tc_vta_scratch_floats(M) floats.
size_t tc_vta_scratch_floats(int64_t M);
void tc_vta(int M, int N, int b, const float* V, int64_t ldv, const float* A, int64_t lda, float* W,
            float* scratch, size_t scratch_floats, unsigned* status, cudaStream_t st);
// C (M x N, ldc) rows r0.. -= V Z on the tensor cores (tcgen05, 3xTF32):
// V is M x b (ldv), Z is b x N (ldz), b <= 64; C 16-byte aligned with ldc*4 a
// multiple of 16 bytes.  scratch holds tc_update_scratch_floats(M, N) floats.
size_t tc_update_scratch_floats(int64_t M, int64_t N);
void tc_update(int M, int N, int b, int r0, const float* V, int64_t ldv, const float* Z, int64_t ldz,
               float* C, int64_t ldc, float* scratch, unsigned* status, cudaStream_t st);
// C rows r0.. -= V Z by tc_update (tensor = true) or the CUDA-core FP32 GEMM.
void update_product(bool tensor, int M, int N, int b, int r0, const float* V, int64_t ldv,
                    const float* Z, int64_t ldz, float* C, int64_t ldc, float* scratch,
                    unsigned* status, cudaStream_t st);
// The CPQR's FP32 products go to the tensor cores unless SKILLS_QR_TC=0.
bool tc_qr_enabled();
// W = V^T A by tc_vta (tensor = true) or the CUDA-core FP32 GEMM; the same
// scratch serves both (split-K partials).
void vta_product(bool tensor, int M, int N, int b, const float* V, int64_t ldv, const float* A,
                 int64_t lda, float* W, float* scratch, size_t scratch_floats, unsigned* status,
                 cudaStream_t st);

// ----------------------------------------------------------- k_trinv.cu --
// M = inv(R11 + perturb*I) for the r x r upper triangle of R (ld); M is r x r
// (ldm), upper triangular, zeros below.  Also ||R11||_inf and ||M||_inf.
template <typename T>
size_t trinv_workspace_bytes(int64_t r);
template <typename T>
void trinv_upper(const T* R, int64_t ld, int64_t r, double perturb, T* M, int64_t ldm,
                 double* norms /* [2] device */, void* work, cudaStream_t st);
template <typename T>
void trmv_upper(const T* M, int64_t ldm, int64_t r, int trans, const double* x, double* y,
                cudaStream_t st);
template <typename T>
int64_t count_rank(const T* R, int64_t ld, int64_t dmin, double abs_thresh, double rel_thresh,
                   int* dev_out, int* host_pinned, cudaStream_t st);

// ------------------------------------------------------------ k_lsqr.cu --
struct LsqrProblem {
    int64_t n = 0, d = 0, nnz = 0;
    // sparse A: CSR rows (A*z) and CSC columns (A^T*u), values in the LSQR
    // storage type: (hi, lo) float pairs for the mixed path, double for FP64
    const int* rp = nullptr; const int* ci = nullptr; const void* cx = nullptr;
    const int* cp = nullptr; const int* ri = nullptr; const void* rx = nullptr;
    const double* cx64 = nullptr; const double* rx64 = nullptr;   // FP64 values
    // dense A: storage-type copy (n x d, lda) and the FP64 original (lda64)
    const void* Ad = nullptr; int64_t lda = 0;
    const double* Ad64 = nullptr; int64_t lda64 = 0;
    // preconditioner: column i of the pivoted set is A(:, cols[i]) scaled by
    // colscale[cols[i]], times M = R11^{-1} (r x r, column-major M and a
    // row-major copy Mrow, both ldm)
    const int* cols = nullptr;
    const double* colscale = nullptr;
    // scale the LSQR products apply to column c of the stored values: colscale
    // when the stored values are A's own, nullptr (1) when they already hold
    // A(:, c) * colscale[c] (the mixed sparse path) or D = I (dense paths)
    const double* opscale = nullptr;
    const void* M = nullptr; const void* Mrow = nullptr; int64_t ldm = 0; int64_t r = 0;
    int precision = SKL_PREC_MIXED;
    // lanes per CSR row (A z) and per CSC column (A^T u); 0 = by the average
    // row / column length
    int lanes_n = 0, lanes_t = 0;
};

struct LsqrResult {
    int flag = 1;
    int64_t it = 0;
    double prof_ms[4] = {0, 0, 0, 0};      // A*z, A^T*u, M*v, M^T*t (profile = 1)
    int64_t prof_launches[4] = {0, 0, 0, 0};
};

size_t lsqr_workspace_bytes(const LsqrProblem& P);
// Solves min || A P1 D M y - b || from y = 0; y (r entries, device).
LsqrResult lsqr_run(const LsqrProblem& P, const double* b, double tol, int64_t max_it, double* y,
                    void* work, unsigned* status, void* host_pinned, cudaStream_t st,
                    int profile = 0, cudaStream_t capture_stream = nullptr);
// One product in isolation with LSQR's storage and arithmetic: y = A x
// (trans 'n', CSR kernel) or y = A^T x ('t', CSC kernel, P.cols = 0..d-1,
// P.r = d).  The stored values are A(:, c) * vscale[c] (vscale nullptr: A's
// own); work holds lsqr_workspace_bytes(P).
void lsqr_product(const LsqrProblem& P, char trans, const double* x, double* y,
                  const double* vscale, void* work, cudaStream_t st);
// Autotuning: the fastest lanes-per-row / per-column of the two sparse
// products on this problem's matrix (P.lanes_n, P.lanes_t).
void tune_lsqr_products(LsqrProblem& P, void* work, cudaStream_t st);
// xfull[cols[i]] = colscale[cols[i]] * (M yv)[i]; scratch holds r float2.
void precond_apply(const LsqrProblem& P, const double* yv, double* xfull, void* scratch,
                   cudaStream_t st);
// out[0] = ||b - A x||, out[1] = ||A^T (b - A x)|| in FP64; r (n) and part
// (512 doubles) are scratch.
void residual_and_backward(const LsqrProblem& P, const double* x, const double* b, double* r,
                           double* part, double* out, cudaStream_t st);
// Refinement of the explicit sketch solution (sparse path).  Direction: with
// rs = b - A x, gm = S rs, dc = M^T D P1^T A^T S^T gm (= Q1^T S rs up to the
// FP32 factor's error), norms[0] = ||gm||, norms[1] = ||dc||; h (n), t (r)
// and part (512) are scratch.  Apply: c += sgn * dc, x = D P1 M c (all d
// entries written), rs = b - A x, *rnorm = ||rs||.
void sketch_refine_direction(const LsqrProblem& P, const int* bptr, const unsigned* bent,
                             const unsigned* hidx, int k, int64_t m, const double* rs, double* gm,
                             double* h, double* t, double* dc, double* part, double* norms,
                             cudaStream_t st);
void sketch_refine_apply(const LsqrProblem& P, double sgn, const double* dc, double* c,
                         const double* b, double* x, double* rs, double* part, double* rnorm,
                         cudaStream_t st);
// (hi, lo) float pairs of the equilibrated values A(:, c) * colscale[c]
// (|value| <= 1, so neither part overflows): CSR entries (column ci[p]) and
// CSC entries (columns by cp).
void split_csr_scaled(const int* ci, const double* cx, int64_t nnz, const double* colscale,
                      float2* out, cudaStream_t st);
void split_csc_scaled(const int* cp, const double* Ax, int64_t d, const double* colscale,
                      float2* out, cudaStream_t st);
// (hi, lo) float pairs of a dense column-major A; sets kStatusRange in
// *status if a nonzero |A_ij| lies outside [2^-100, 2^100].
constexpr unsigned kStatusRange = 32u;
void split_dense(const double* A, int64_t lda, int64_t n, int64_t d, float2* out,
                 unsigned* status, cudaStream_t st);
// x[0..n) += a[0..n)
void vec_add(double* x, const double* a, int64_t n, cudaStream_t st);
// Columns r..r2-1 of the upper-triangular M (column-major, ldm) become the
// unit vectors e_j (zeros above the diagonal, 1 on it).
template <typename T>
void extend_identity(T* Mc, int64_t ldm, int64_t r, int64_t r2, cudaStream_t st);
template <typename T>
void transpose_upper(const T* Mc, int64_t ldm, int64_t r, T* Mr, cudaStream_t st);

// ----------------------------------------------------------- hashing.cpp --
// Host generator compatible with the C library's rand() (glibc TYPE_3).
void rng_srand(uint32_t seed);
// Draws the s-hashing matrix of sparse_helpers.cpp:90-116 from the library
// stream: hidx[i*k+j] = row | (sign < 0 ? 0x80000000 : 0).
void gen_hash_packed(int64_t m, int64_t n, int64_t k, uint32_t* hidx);
// n random signs (+-1) as in gen_scaled_rand_signs (dense_helpers.cpp:7-16).
void gen_signs(int64_t n, double* D);
// The m rows random_sample keeps of N (dense_helpers.cpp:19-39): the first m
// entries of 0..N-1 after select_k_from_n's partial Fisher-Yates shuffle
// (sparse_helpers.cpp:74-86) on the library stream.  Caller holds the lock.
void gen_subsample(int64_t N, int64_t m, uint32_t* rows);
// Leaves the library stream where HQRRP leaves the C library's: srand(12),
// then the rand() calls of Marsaglia's polar method for rows*cols normals.
void rng_hqrrp_advance(int64_t rows, int64_t cols);
void rng_lock();
void rng_unlock();

}  // namespace skl
