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
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
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

// Caller holds the lock (rng_lock).
void gen_hash_packed(int64_t m, int64_t n, int64_t k, uint32_t* hidx)
{
    std::vector<uint32_t> perm((size_t)m);
    for (int64_t i = 0; i < m; ++i) perm[(size_t)i] = (uint32_t)i;
    uint32_t* pa = perm.data();
    if (k == 1) {
        const uint32_t mm = (uint32_t)m;
        for (int64_t i = 0; i < n; ++i) {
            uint32_t t = g_rng.next() % mm;
            uint32_t a = pa[t];
            pa[t] = pa[0];
            pa[0] = a;
            hidx[i] = a;
        }
    } else {
        for (int64_t i = 0; i < n; ++i) {
            uint32_t* out = hidx + i * k;
            for (int64_t j = 0; j < k; ++j) {
                uint32_t t = (uint32_t)(g_rng.next() % (uint32_t)(m - j)) + (uint32_t)j;
                uint32_t a = pa[t];
                pa[t] = pa[j];
                pa[j] = a;
                out[j] = a;
            }
        }
    }
    const int64_t nk = n * k;
    for (int64_t q = 0; q < nk; ++q)
        if ((g_rng.next() & 1u) == 0u) hidx[q] |= 0x80000000u;   // rand()%2 == 0 -> -1
}

// Caller holds the lock.
void gen_signs(int64_t n, double* D)
{
    for (int64_t i = 0; i < n; ++i) D[i] = (g_rng.next() & 1u) ? 1.0 : -1.0;
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
