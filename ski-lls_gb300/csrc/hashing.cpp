// hashing.cpp -- the s-hashing matrix drawn exactly as the reference draws it.
//
// The reference calls the C library's rand() (glibc's TYPE_3 additive
// feedback generator: 31 state words, separation 3, Lehmer-seeded, 310 warm-up
// outputs, output = word >> 1) from gen_hashing_matrix / select_k_from_n
// (src/sparse_helpers.cpp:74-116) and gen_scaled_rand_signs
// (src/dense_helpers.cpp:7-16).  The library keeps its own stream with the
// same recurrence so that, for the same seed, rows and signs are bit-identical
// to the reference; a fresh process starts at seed 1 like the C library.
//
// Column i of S (row i of A) takes k distinct rows from a partial
// Fisher-Yates shuffle of a permutation array that persists across columns;
// all n*k signs are drawn after all rows.  The shuffle is inherently serial,
// so it runs on the host while the device copies and converts A.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <array>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "skl_internal.hpp"

namespace skl {

namespace {

struct Rng {
    uint32_t s[31];
    int f = 3, r = 0;

    void seed(uint32_t sd)
    {
        if (sd == 0) sd = 1;
        int32_t word = (int32_t)sd;
        s[0] = (uint32_t)word;
        for (int i = 1; i < 31; ++i) {
            // 16807 * word mod (2^31 - 1), Schrage's decomposition
            long hi = word / 127773;
            long lo = word % 127773;
            long w = 16807 * lo - 2836 * hi;
            if (w < 0) w += 2147483647;
            word = (int32_t)w;
            s[i] = (uint32_t)word;
        }
        f = 3;
        r = 0;
        for (int i = 0; i < 310; ++i) next();
    }

    inline uint32_t next()
    {
        uint32_t v = s[f] + s[r];
        s[f] = v;
        if (++f == 31) f = 0;
        if (++r == 31) r = 0;
        return v >> 1;
    }

    // The state after L more draws, without drawing them.  The words obey
    // x_t = x_{t-31} + x_{t-3} (mod 2^32), so x_{t+L} is a fixed Z/2^32
    // combination of the current window x_{t-31..t-1}: the coefficients of
    // X^L mod (X^31 - X^28 - 1), formed by square-and-multiply.
    Rng jumped(uint64_t L) const
    {
        using Poly = std::array<uint32_t, 31>;
        auto mulmod = [](const Poly& a, const Poly& b) {
            uint32_t prod[61] = {0};
            for (int i = 0; i < 31; ++i)
                for (int j = 0; j < 31; ++j) prod[i + j] += a[(size_t)i] * b[(size_t)j];
            // X^e = X^(e-3) + X^(e-31) for e >= 31, highest degree first
            for (int e = 60; e >= 31; --e) {
                prod[e - 3] += prod[e];
                prod[e - 31] += prod[e];
                prod[e] = 0;
            }
            Poly r{};
            for (int i = 0; i < 31; ++i) r[(size_t)i] = prod[i];
            return r;
        };
        Poly acc{}, base{};
        acc[0] = 1;    // X^0
        base[1] = 1;   // X^1
        for (uint64_t e = L; e; e >>= 1) {
            if (e & 1) acc = mulmod(acc, base);
            base = mulmod(base, base);
        }
        uint32_t w[31];   // current window, oldest first
        for (int t = 0; t < 31; ++t) w[t] = s[(f + t) % 31];
        Rng out;
        Poly c = acc;     // X^(L + t) mod P for t = 0, 1, ...
        for (int t = 0; t < 31; ++t) {
            uint32_t v = 0;
            for (int u = 0; u < 31; ++u) v += c[(size_t)u] * w[u];
            out.s[(3 + t) % 31] = v;
            // c <- X c mod P
            const uint32_t top = c[30];
            for (int u = 30; u > 0; --u) c[(size_t)u] = c[(size_t)u - 1];
            c[0] = 0;
            c[28] += top;
            c[0] += top;
        }
        out.f = 3;
        out.r = 0;
        return out;
    }
};

std::mutex g_mu;
Rng g_rng;
bool g_seeded = false;

void ensure_seeded()
{
    if (!g_seeded) {
        g_rng.seed(1);
        g_seeded = true;
    }
}

}  // namespace

void rng_lock()
{
    g_mu.lock();
    ensure_seeded();
}

void rng_unlock() { g_mu.unlock(); }

void rng_srand(uint32_t seed)
{
    std::lock_guard<std::mutex> lk(g_mu);
    g_rng.seed(seed);
    g_seeded = true;
}

// x mod d for 32-bit x and d >= 1 with the precomputed M = floor((2^64 - 1) / d) + 1
// (the direct remainder computation of Lemire, Kaser and Kurz, "Faster
// remainder by direct computation", 2019): exact for every 32-bit x, two
// multiplies instead of a division.
static inline uint32_t fastmod_u32(uint32_t x, uint64_t M, uint32_t d)
{
    const uint64_t low = M * x;
    return (uint32_t)(((unsigned __int128)low * d) >> 64);
}

// The serial Fisher-Yates swaps over precomputed targets (tt[s]: target of
// draw s, sign in bit 31).  For small k the head of the array (positions
// 0..k-1, the only positions a draw writes besides its target) stays in
// registers, so a draw costs one load and one store of the array.
template <int K>
static void swaps_head(uint32_t* pa, const uint32_t* tp, int64_t n, uint32_t* hidx)
{
    uint32_t h[K];
    for (int j = 0; j < K; ++j) h[j] = pa[j];
    for (int64_t i = 0; i < n; ++i) {
        const uint32_t* w = tp + i * K;
        uint32_t* out = hidx + i * K;
#pragma GCC unroll 4
        for (int j = 0; j < K; ++j) {
            const uint32_t t = w[j] & 0x7fffffffu;
            uint32_t a;
            if (t < (uint32_t)K) {   // t >= j: both ends in the head
                a = h[0];
                for (int q = 1; q < K; ++q) a = (t == (uint32_t)q) ? h[q] : a;
                for (int q = 0; q < K; ++q) h[q] = (t == (uint32_t)q) ? h[j] : h[q];
            } else {
                a = pa[t];
                pa[t] = h[j];
            }
            h[j] = a;
            out[j] = a | (w[j] & 0x80000000u);
        }
    }
    for (int j = 0; j < K; ++j) pa[j] = h[j];
}

// Draw counts below this run on the calling thread alone (thread start-up
// costs more than the parallel draws save there; measured: 2^15 is better
// than 2^17 to 2^20 on the 512-problem batch).
constexpr int64_t kHashSerialMax = (int64_t)1 << 15;

// Caller holds the lock (rng_lock).  The stream gives n*k row draws, then
// n*k sign draws.  Only the Fisher-Yates swaps are serial; the draws
// themselves are not, so for large n*k worker threads start from the states
// jumped to their chunk of both draw sequences and turn their words into swap
// targets t = word % (m - j) + j with the sign bit, and this thread then runs
// the swaps over the precomputed targets.
void gen_hash_packed(int64_t m, int64_t n, int64_t k, uint32_t* hidx)
{
    const int64_t nk = n * k;
    std::vector<uint32_t> perm((size_t)m);
    for (int64_t i = 0; i < m; ++i) perm[(size_t)i] = (uint32_t)i;
    uint32_t* pa = perm.data();
    if (nk < kHashSerialMax) {
        // a local copy of the generator (the global one would be reloaded and
        // stored around every draw: the output writes may alias it)
        Rng g = g_rng;
        std::vector<uint64_t> mg((size_t)k);
        for (int64_t j = 0; j < k; ++j) mg[(size_t)j] = UINT64_C(0xFFFFFFFFFFFFFFFF) / (uint64_t)(m - j) + 1;
        for (int64_t i = 0; i < n; ++i) {
            uint32_t* out = hidx + i * k;
            for (int64_t j = 0; j < k; ++j) {
                uint32_t t = fastmod_u32(g.next(), mg[(size_t)j], (uint32_t)(m - j)) + (uint32_t)j;
                uint32_t a = pa[t];
                pa[t] = pa[j];
                pa[j] = a;
                out[j] = a;
            }
        }
        for (int64_t q = 0; q < nk; ++q)
            if ((g.next() & 1u) == 0u) hidx[q] |= 0x80000000u;   // rand()%2 == 0 -> -1
        g_rng = g;
        return;
    }
    // tt[s]: swap target of draw s, with the sign in bit 31 (set = -1); left
    // uninitialised here, every entry is written once by the worker whose chunk
    // holds it (the pages are first touched by those workers)
    std::unique_ptr<uint32_t[]> tt(new uint32_t[(size_t)nk]);
    // the divisors m - j and their remainder constants
    std::vector<uint64_t> magic((size_t)k);
    for (int64_t j = 0; j < k; ++j) magic[(size_t)j] = UINT64_C(0xFFFFFFFFFFFFFFFF) / (uint64_t)(m - j) + 1;
    const unsigned hw = std::thread::hardware_concurrency();
    const int64_t nthr = std::max<int64_t>(1, std::min<int64_t>({(int64_t)(hw ? hw : 4), 16, nk >> 14}));
    const int64_t chunk = (nk + nthr - 1) / nthr;
    const Rng base = g_rng;
    auto work = [&](int64_t c) {
        const int64_t s0 = c * chunk, s1 = std::min(nk, s0 + chunk);
        if (s0 >= s1) return;
        Rng rows = base.jumped((uint64_t)s0);
        Rng signs = base.jumped((uint64_t)(nk + s0));
        int64_t j = s0 % k;
        uint32_t* out = tt.get();
        for (int64_t s = s0; s < s1; ++s) {
            const uint32_t d = (uint32_t)(m - j);
            const uint32_t t = fastmod_u32(rows.next(), magic[(size_t)j], d) + (uint32_t)j;
            const uint32_t neg = (signs.next() & 1u) == 0u ? 0x80000000u : 0u;   // rand()%2 == 0 -> -1
            out[s] = t | neg;
            if (++j == k) j = 0;
        }
    };
    std::vector<std::thread> pool;
    for (int64_t c = 1; c < nthr; ++c) pool.emplace_back(work, c);
    work(0);
    for (auto& t : pool) t.join();
    const uint32_t* tp = tt.get();
    if (k == 1) {
        swaps_head<1>(pa, tp, n, hidx);
    } else if (k == 2) {
        swaps_head<2>(pa, tp, n, hidx);
    } else if (k == 3) {
        swaps_head<3>(pa, tp, n, hidx);
    } else if (k == 4) {
        swaps_head<4>(pa, tp, n, hidx);
    } else {
        int64_t j = 0;
        for (int64_t s = 0; s < nk; ++s) {
            const uint32_t w = tp[s], t = w & 0x7fffffffu;
            const uint32_t a = pa[t];
            pa[t] = pa[j];
            pa[j] = a;
            hidx[s] = a | (w & 0x80000000u);
            if (++j == k) j = 0;
        }
    }
    g_rng = base.jumped((uint64_t)(2 * nk));   // the stream continues after both draw sequences
}

// Caller holds the lock.
void gen_signs(int64_t n, double* D)
{
    for (int64_t i = 0; i < n; ++i) D[i] = (g_rng.next() & 1u) ? 1.0 : -1.0;
}

// Caller holds the lock.  Step i draws t = rand() % (N - i) + i and swaps
// entries i and t of the index array; entry i is final after step i.
void gen_subsample(int64_t N, int64_t m, uint32_t* rows)
{
    std::vector<uint32_t> idx((size_t)N);
    for (int64_t i = 0; i < N; ++i) idx[(size_t)i] = (uint32_t)i;
    for (int64_t i = 0; i < m; ++i) {
        const uint32_t t = (uint32_t)(g_rng.next() % (uint32_t)(N - i)) + (uint32_t)i;
        const uint32_t a = idx[t];
        idx[t] = idx[(size_t)i];
        idx[(size_t)i] = a;
        rows[i] = a;
    }
}

// NoFLA_Normal_random_matrix / NoFLA_Normal_random_number
// (hqrrp/lapack_compatible_sources/NoFLA_HQRRP_WY_blk_var4_skint.c:584-624):
// pairs (c1, c2) uniform in (-1,1)^2 are drawn until 0 < c1^2+c2^2 < 1; each
// accepted pair yields two normals.  Only the number of rand() calls matters.
void rng_hqrrp_advance(int64_t rows, int64_t cols)
{
    std::lock_guard<std::mutex> lk(g_mu);
    g_rng.seed(12);
    g_seeded = true;
    const int64_t count = rows * cols;
    const double rmax = 2147483647.0;
    for (int64_t q = 0; q < count; q += 2) {
        double a;
        do {
            const double c1 = -1.0 + 2.0 * ((double)g_rng.next() / rmax);
            const double c2 = -1.0 + 2.0 * ((double)g_rng.next() / rmax);
            const double p1 = c1 * c1;
            const double p2 = c2 * c2;
            a = p1 + p2;
        } while (a == 0 || a >= 1);
    }
}

}  // namespace skl

extern "C" void skl_srand(uint32_t seed) { skl::rng_srand(seed); }

extern "C" skl_status skl_subsample_rows(int64_t N, int64_t m, int seed_mode, uint32_t seed,
                                         int64_t* rows)
{
    if (N <= 0 || m < 0 || m > N || N > 0x7fffffff || (m > 0 && !rows)) return SKL_ERR_INVALID;
    std::vector<uint32_t> r((size_t)m);
    if (seed_mode) skl::rng_srand(seed);
    skl::rng_lock();
    skl::gen_subsample(N, m, r.data());
    skl::rng_unlock();
    for (int64_t i = 0; i < m; ++i) rows[i] = (int64_t)r[(size_t)i];
    return SKL_OK;
}

extern "C" skl_status skl_hash_generate(int64_t m, int64_t n, int64_t k, int seed_mode,
                                        uint32_t seed, int64_t* rows, double* vals)
{
    if (m <= 0 || n < 0 || k < 1 || k > m || m > 0x7fffffff || !rows || !vals)
        return SKL_ERR_INVALID;
    std::vector<uint32_t> h((size_t)(n * k));
    skl::rng_lock();
    if (seed_mode) {
        skl::rng_unlock();
        skl::rng_srand(seed);
        skl::rng_lock();
    }
    skl::gen_hash_packed(m, n, k, h.data());
    skl::rng_unlock();
    const double v = 1.0 / std::sqrt((double)k);
    for (int64_t q = 0; q < n * k; ++q) {
        rows[q] = (int64_t)(h[(size_t)q] & 0x7fffffffu);
        vals[q] = (h[(size_t)q] & 0x80000000u) ? -v : v;
    }
    return SKL_OK;
}
