// k_format.cu -- device-side sparse format work for the solve path.
//
//  * CSC input validation and narrowing (64-bit cs_dl indices -> int32),
//  * exclusive scans,
//  * a stable LSD radix sort of 32-bit keys with 32-bit payloads, used to build
//    a CSR copy of A whose rows keep column order (so every SpMV sums in a
//    fixed order and results are bitwise reproducible) and the bucket lists of
//    the hashing matrix S (rows of S with their source rows in order).
#include "skl_internal.hpp"
#include "launch.cuh"
#include "common.cuh"

namespace skl {

// ------------------------------------------------------------ validation --
// Narrow Ap/Ai to int32 and check the CSC structure: Ap[0] = 0, Ap
// non-decreasing, Ap[n] = nnz, 0 <= Ai < m.  Values are checked for finiteness.
__global__ void k_csc_narrow_colptr(const int64_t* __restrict__ Ap, int64_t ncol, int64_t nnz,
                                    int* __restrict__ cp, unsigned* __restrict__ bad)
{
    pdl_wait();
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j <= ncol;
         j += (int64_t)gridDim.x * blockDim.x) {
        int64_t v = Ap[j];
        bool ok = v >= 0 && v <= nnz;
        if (j == 0) ok = ok && v == 0;
        if (j == ncol) ok = ok && v == nnz;
        if (j > 0) ok = ok && Ap[j - 1] <= v;
        if (!ok) atomicOr(bad, 1u);
        cp[j] = (int)v;
    }
}

__global__ void k_csc_narrow_rows(const int64_t* __restrict__ Ai, const double* __restrict__ Ax,
                                  int64_t nnz, int64_t nrow, int* __restrict__ ri,
                                  unsigned* __restrict__ bad)
{
    pdl_wait();
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nnz;
         p += (int64_t)gridDim.x * blockDim.x) {
        int64_t r = Ai[p];
        if (r < 0 || r >= nrow) {
            atomicOr(bad, 2u);
            r = 0;
        }
        if (!isfinite(Ax[p])) atomicOr(bad, 4u);
        ri[p] = (int)r;
    }
}

// col index of every nonzero (CSC order) from the column pointers.
__global__ void k_expand_colptr(const int* __restrict__ cp, int ncol, int* __restrict__ colof)
{
    pdl_wait();
    int j = blockIdx.x;
    if (j >= ncol) return;
    for (int p = cp[j] + threadIdx.x; p < cp[j + 1]; p += blockDim.x) colof[p] = j;
}

__global__ void k_iota(unsigned* __restrict__ v, int64_t n)
{
    pdl_wait();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        v[i] = (unsigned)i;
}

// ------------------------------------------------------------------ scan --
// Exclusive scan of int32 counts into int32 offsets; out has n+1 entries and
// out[n] = total.  Three-phase: per-tile scan, scan of tile sums, fix-up.
constexpr int kScanThreads = 512;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void k_scan_tiles(const int* __restrict__ in, int64_t n, int* __restrict__ out,
                             int* __restrict__ tile_sums)
{
    pdl_wait();
    __shared__ int s_warp[kScanThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int v[kScanItems];
    int tsum = 0;
#pragma unroll
    for (int t = 0; t < kScanItems; ++t) {
        int64_t i = base + t;
        v[t] = (i < n) ? in[i] : 0;
        tsum += v[t];
    }
    // warp inclusive scan of per-thread sums
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int incl = tsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) s_warp[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        int w = (lane < kScanThreads / 32) ? s_warp[lane] : 0;
        int wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += y;
        }
        if (lane < kScanThreads / 32) s_warp[lane] = wi - w;
    }
    __syncthreads();
    int run = s_warp[wid] + incl - tsum;
#pragma unroll
    for (int t = 0; t < kScanItems; ++t) {
        int64_t i = base + t;
        if (i < n) out[i] = run;
        run += v[t];
    }
    if (threadIdx.x == kScanThreads - 1) tile_sums[blockIdx.x] = run;
}

__global__ void k_scan_add(int* __restrict__ out, int64_t n, const int* __restrict__ tile_off)
{
    pdl_wait();
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    const int add = tile_off[blockIdx.x];
    for (int t = threadIdx.x; t < kScanTile; t += blockDim.x) {
        int64_t i = base + t;
        if (i < n) out[i] += add;
    }
}

__global__ void k_set_last(int* out, int64_t n, const int* tile_sums_scanned, int ntiles)
{
    pdl_wait();
    // total = exclusive prefix of the last tile + its sum (stored at index ntiles)
    out[n] = tile_sums_scanned[ntiles];
}

// Scratch needed by scan_exclusive for n items.
size_t scan_scratch_ints(int64_t n)
{
    int64_t tiles = (n + kScanTile - 1) / kScanTile;
    if (tiles <= 1) return 4;
    return (size_t)(2 * (tiles + 1)) + scan_scratch_ints(tiles + 1);
}

void scan_exclusive(const int* in, int64_t n, int* out, int* scratch, cudaStream_t st)
{
    int64_t tiles = (n + kScanTile - 1) / kScanTile;
    if (tiles < 1) tiles = 1;
    int* sums = scratch;                 // tiles+1
    int* sums_scan = scratch + tiles + 1;  // tiles+1
    launch_k(k_scan_tiles, (unsigned)tiles, kScanThreads, 0, st, in, n, out, sums);
    SKL_LAUNCHED();
    if (tiles == 1) {
        // sums[0] is the total
        cudaMemcpyAsync(out + n, sums, sizeof(int), cudaMemcpyDeviceToDevice, st);
        return;
    }
    // scan the tile sums (tiles entries) -> sums_scan[0..tiles], sums_scan[tiles] = total
    scan_exclusive(sums, tiles, sums_scan, scratch + 2 * (tiles + 1), st);
    launch_k(k_scan_add, (unsigned)tiles, kScanThreads, 0, st, out, n, sums_scan);
    SKL_LAUNCHED();
    launch_k(k_set_last, 1, 1, 0, st, out, n, sums_scan, (int)tiles);
    SKL_LAUNCHED();
}

// ------------------------------------------------------------ radix sort --
// Stable LSD radix sort of (key, payload) pairs, 8 bits per pass.
constexpr int kRsThreads = 256;
constexpr int kRsChunks = 32;                    // warp-chunks of 32 items per tile
constexpr int kRsTile = kRsChunks * 32;          // 1024 items per tile
constexpr int kRsBins = 256;

__global__ void k_rs_hist(const unsigned* __restrict__ keys, int64_t n, int shift,
                          int* __restrict__ hist /* [bins][tiles] */, int tiles)
{
    pdl_wait();
    __shared__ int h[kRsBins];
    for (int b = threadIdx.x; b < kRsBins; b += blockDim.x) h[b] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kRsTile;
    for (int t = threadIdx.x; t < kRsTile; t += blockDim.x) {
        int64_t i = base + t;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 0xff], 1);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < kRsBins; b += blockDim.x) hist[(int64_t)b * tiles + blockIdx.x] = h[b];
}

__global__ void k_rs_scatter(const unsigned* __restrict__ keys, const unsigned* __restrict__ vals,
                             int64_t n, int shift, const int* __restrict__ offs /* scanned hist */,
                             int tiles, unsigned* __restrict__ keys_out,
                             unsigned* __restrict__ vals_out)
{
    pdl_wait();
    __shared__ int cnt[kRsBins][kRsChunks + 1];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
    for (int i = threadIdx.x; i < kRsBins * (kRsChunks + 1); i += blockDim.x) (&cnt[0][0])[i] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kRsTile;
    // pass 1: per chunk digit counts
    for (int c = wid; c < kRsChunks; c += nw) {
        int64_t i = base + (int64_t)c * 32 + lane;
        bool valid = i < n;
        unsigned dig = valid ? ((keys[i] >> shift) & 0xff) : 0xffffffffu;
        unsigned peers = __match_any_sync(0xffffffffu, dig);
        if (valid && lane == (__ffs(peers) - 1)) cnt[dig][c] = __popc(peers);
    }
    __syncthreads();
    // exclusive scan over chunks for each digit, plus the tile's global offset
    for (int d = threadIdx.x; d < kRsBins; d += blockDim.x) {
        int run = offs[(int64_t)d * tiles + blockIdx.x];
        for (int c = 0; c < kRsChunks; ++c) {
            int v = cnt[d][c];
            cnt[d][c] = run;
            run += v;
        }
    }
    __syncthreads();
    for (int c = wid; c < kRsChunks; c += nw) {
        int64_t i = base + (int64_t)c * 32 + lane;
        bool valid = i < n;
        unsigned key = valid ? keys[i] : 0u;
        unsigned dig = valid ? ((key >> shift) & 0xff) : 0xffffffffu;
        unsigned peers = __match_any_sync(0xffffffffu, dig);
        if (valid) {
            unsigned lt = (1u << lane) - 1u;
            int dst = cnt[dig][c] + __popc(peers & lt);
            keys_out[dst] = key;
            vals_out[dst] = vals[i];
        }
    }
}

size_t radix_sort_scratch_ints(int64_t n)
{
    int64_t tiles = (n + kRsTile - 1) / kRsTile;
    if (tiles < 1) tiles = 1;
    int64_t h = tiles * kRsBins;
    return (size_t)(2 * (h + 1)) + scan_scratch_ints(h);
}

// Sorts (keys, vals) stably by the low `bits` bits of keys.  keys_tmp/vals_tmp
// are buffers of n entries; the result ends in keys/vals.
void radix_sort_pairs(unsigned* keys, unsigned* vals, unsigned* keys_tmp, unsigned* vals_tmp,
                      int64_t n, int bits, int* scratch, cudaStream_t st)
{
    if (n <= 0) return;
    int64_t tiles = (n + kRsTile - 1) / kRsTile;
    int64_t h = tiles * kRsBins;
    int* hist = scratch;
    int* offs = scratch + (h + 1);
    int* sscr = scratch + 2 * (h + 1);
    unsigned *ka = keys, *va = vals, *kb = keys_tmp, *vb = vals_tmp;
    int passes = (bits + 7) / 8;
    for (int p = 0; p < passes; ++p) {
        int shift = 8 * p;
        launch_k(k_rs_hist, (unsigned)tiles, kRsThreads, 0, st, ka, n, shift, hist, (int)tiles);
        SKL_LAUNCHED();
        scan_exclusive(hist, h, offs, sscr, st);
        launch_k(k_rs_scatter, (unsigned)tiles, kRsThreads, 0, st, ka, va, n, shift, offs, (int)tiles, kb, vb);
        SKL_LAUNCHED();
        unsigned* t = ka; ka = kb; kb = t;
        t = va; va = vb; vb = t;
    }
    if (ka != keys) {
        cudaMemcpyAsync(keys, ka, n * sizeof(unsigned), cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(vals, va, n * sizeof(unsigned), cudaMemcpyDeviceToDevice, st);
    }
}

int bits_for(int64_t maxval)
{
    int b = 1;
    while (b < 32 && ((int64_t)1 << b) <= maxval) ++b;
    return b;
}

// ------------------------------------------------------------- CSR build --
__global__ void k_count_rows(const int* __restrict__ ri, int64_t nnz, int* __restrict__ cnt)
{
    pdl_wait();
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < nnz;
         p += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&cnt[ri[p]], 1);
}

__global__ void k_csr_gather(const unsigned* __restrict__ perm, int64_t nnz,
                             const int* __restrict__ colof, const double* __restrict__ Ax,
                             int* __restrict__ ci, double* __restrict__ cx)
{
    pdl_wait();
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nnz;
         q += (int64_t)gridDim.x * blockDim.x) {
        unsigned p = perm[q];
        ci[q] = colof[p];
        cx[q] = Ax[p];
    }
}

// ---------------------------------------------------------- host drivers --
static unsigned grid_for(int64_t n, int threads, int cap = 152 * 16)
{
    int64_t g = (n + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (unsigned)g;
}

void csc_narrow(const int64_t* Ap, const int64_t* Ai, const double* Ax, int64_t nrow, int64_t ncol,
                int64_t nnz, int* cp, int* ri, unsigned* bad, cudaStream_t st)
{
    launch_k(k_csc_narrow_colptr, grid_for(ncol + 1, 256), 256, 0, st, Ap, ncol, nnz, cp, bad);
    SKL_LAUNCHED();
    if (nnz > 0) {
        launch_k(k_csc_narrow_rows, grid_for(nnz, 256), 256, 0, st, Ai, Ax, nnz, nrow, ri, bad);
        SKL_LAUNCHED();
    }
}

// Workspace (ints) for build_csr: see the layout in build_csr.
size_t build_csr_scratch_ints(int64_t nrow, int64_t nnz)
{
    size_t s = (size_t)(nrow + 1) + 5 * (size_t)nnz;
    size_t a = scan_scratch_ints(nrow + 1), b = radix_sort_scratch_ints(nnz);
    return s + (a > b ? a : b);
}

void build_csr(const int* cp, const int* ri, const double* Ax, int64_t nrow, int64_t ncol,
               int64_t nnz, int* rp, int* ci, double* cx, int* scratch, cudaStream_t st)
{
    int* cnt = scratch;                                 // nrow+1
    unsigned* keys = (unsigned*)(cnt + nrow + 1);       // nnz
    unsigned* perm = keys + nnz;                        // nnz
    unsigned* ktmp = perm + nnz;                        // nnz
    unsigned* vtmp = ktmp + nnz;                        // nnz
    int* colof = (int*)(vtmp + nnz);                    // nnz
    int* rest = colof + nnz;
    cudaMemsetAsync(cnt, 0, (nrow + 1) * sizeof(int), st);
    if (nnz > 0) {
        launch_k(k_count_rows, grid_for(nnz, 256), 256, 0, st, ri, nnz, cnt);
        SKL_LAUNCHED();
    }
    scan_exclusive(cnt, nrow, rp, rest, st);
    if (nnz == 0) return;
    cudaMemcpyAsync(keys, ri, nnz * sizeof(int), cudaMemcpyDeviceToDevice, st);
    launch_k(k_iota, grid_for(nnz, 256), 256, 0, st, perm, nnz);
    SKL_LAUNCHED();
    launch_k(k_expand_colptr, (unsigned)ncol, 128, 0, st, cp, (int)ncol, colof);
    SKL_LAUNCHED();
    radix_sort_pairs(keys, perm, ktmp, vtmp, nnz, bits_for(nrow - 1), rest, st);
    launch_k(k_csr_gather, grid_for(nnz, 256), 256, 0, st, perm, nnz, colof, Ax, ci, cx);
    SKL_LAUNCHED();
}

// ------------------------------------------------------- hash buckets --
// hidx[i*k+t] = row h of S | sign bit (bit 31 set for -1).  Buckets: for each
// h, the packed (i | sign) entries in increasing i.
__global__ void k_hash_keys(const unsigned* __restrict__ hidx, int64_t nk, int k,
                            unsigned* __restrict__ keys, unsigned* __restrict__ vals,
                            int* __restrict__ cnt)
{
    pdl_wait();
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nk;
         q += (int64_t)gridDim.x * blockDim.x) {
        unsigned e = hidx[q];
        unsigned h = e & 0x7fffffffu;
        keys[q] = h;
        vals[q] = (unsigned)(q / k) | (e & 0x80000000u);
        atomicAdd(&cnt[h], 1);
    }
}

// Every hashed row must lie in [0, m): the bucket build and the sketch use
// them as addresses.  Flags bit 16 of *status otherwise.
__global__ void k_check_hash_rows(const unsigned* __restrict__ hidx, int64_t nk, unsigned m,
                                  unsigned* __restrict__ status)
{
    pdl_wait();
    bool bad = false;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nk;
         q += (int64_t)gridDim.x * blockDim.x)
        bad = bad || (hidx[q] & 0x7fffffffu) >= m;
    if (bad) atomicOr(status, 16u);
}

void check_hash_rows(const unsigned* hidx, int64_t nk, int64_t m, unsigned* status, cudaStream_t st)
{
    if (nk <= 0) return;
    launch_k(k_check_hash_rows, grid_for(nk, 256), 256, 0, st, hidx, nk, (unsigned)m, status);
    SKL_LAUNCHED();
}

size_t build_buckets_scratch_ints(int64_t m, int64_t nk)
{
    size_t s = (size_t)(m + 1) + 4 * (size_t)nk;
    size_t a = scan_scratch_ints(m + 1), b = radix_sort_scratch_ints(nk);
    return s + (a > b ? a : b);
}

void build_buckets(const unsigned* hidx, int64_t n, int k, int64_t m, int* bptr, unsigned* bent,
                   int* scratch, cudaStream_t st)
{
    int64_t nk = n * k;
    int* cnt = scratch;
    unsigned* keys = (unsigned*)(cnt + m + 1);
    unsigned* ktmp = keys + nk;
    unsigned* vtmp = ktmp + nk;
    int* rest = (int*)(vtmp + nk);
    cudaMemsetAsync(cnt, 0, (m + 1) * sizeof(int), st);
    launch_k(k_hash_keys, grid_for(nk, 256), 256, 0, st, hidx, nk, k, keys, bent, cnt);
    SKL_LAUNCHED();
    scan_exclusive(cnt, m, bptr, rest, st);
    radix_sort_pairs(keys, bent, ktmp, vtmp, nk, bits_for(m - 1), rest, st);
}

}  // namespace skl
