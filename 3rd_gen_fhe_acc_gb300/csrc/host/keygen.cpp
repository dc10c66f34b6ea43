// keygen.cpp -- seeded key generation, encryption and decryption on the host.
//
// The reference draws its randomness from std::default_random_engine seeded by
// std::random_device (src/RNG.cpp:3-36), which is neither reproducible nor the same
// across standard libraries. Here every object is drawn from its own SplitMix64
// stream keyed by (seed, object kind, object index), so a seed gives the same
// words on every machine and for any thread count. The distributions are the
// reference's: uniform mod q / mod Q, ternary {-1, 0, 1} secrets with the
// reference's rejection bounds, and a normal variate (sigma 3.19) truncated
// toward zero and reduced '% bound' (RNG_norm::generate_norm, include/RNG.h:27,
// src/RNG.cpp:19-36), sampled from an integer
// cumulative table (gauss_cdt.inc).
#include "host_math.hpp"
#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "gauss_cdt.inc"

namespace fheacc {
namespace host {

enum : uint64_t {
    TAG_LWE_SK = 1, TAG_RLWE_SK = 2, TAG_BTKEY = 3, TAG_LWE_KS = 4,
    TAG_SUBS = 5, TAG_LWE_ENC = 6, TAG_RLWE_ENC = 7, TAG_RGSW_ENC = 8,
};

static inline uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

// SplitMix64 stream.
struct Rng {
    uint64_t s;
    Rng(uint64_t seed, uint64_t tag, uint64_t idx)
    {
        s = mix64(seed + 0x9E3779B97F4A7C15ULL);
        s = mix64(s ^ (tag * 0xD1B54A32D192ED03ULL));
        s = mix64(s ^ (idx + 0x632BE59BD9B4E019ULL));
    }
    uint64_t next()
    {
        s += 0x9E3779B97F4A7C15ULL;
        return mix64(s);
    }
    // uniform in [0, m), by rejection on the top bits
    uint64_t uniform(uint64_t m)
    {
        if (m <= 1) return 0;
        int bits = 64 - __builtin_clzll(m - 1);
        for (;;) {
            uint64_t x = bits == 64 ? next() : next() >> (64 - bits);
            if (x < m) return x;
        }
    }
    int64_t ternary() { return (int64_t)uniform(3) - 1; }
    // RNG_norm::generate_norm(bound), include/RNG.h:27, src/RNG.cpp:19-36
    int64_t gauss(uint64_t bound)
    {
        uint64_t u = next();
        int i = 0;
        while (i < 2 * FHEACC_GAUSS_K && u >= kGaussCdt[i]) i++;
        int64_t v = (int64_t)i - FHEACC_GAUSS_K;
        return v % (int64_t)bound;
    }
};

static inline uint64_t mod_signed(int64_t v, uint64_t m)
{
    int64_t r = v % (int64_t)m;
    return (uint64_t)(r < 0 ? r + (int64_t)m : r);
}

template <class F>
static void parallel_for(size_t count, int threads, F f)
{
    if (threads <= 0) threads = (int)std::thread::hardware_concurrency();
    if (threads < 1) threads = 1;
    if ((size_t)threads > count) threads = (int)std::max<size_t>(count, 1);
    std::atomic<size_t> next(0);
    auto work = [&]() {
        for (;;) {
            size_t i = next.fetch_add(1);
            if (i >= count) break;
            f(i);
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; t++) pool.emplace_back(work);
    work();
    for (auto &th : pool) th.join();
}

// RLWE_encrypt of the zero plaintext (RLWE.cpp:324-344): a uniform, e noise,
// both moved to the NTT domain, b = a*s + e. out = a[N], b[N].
static void rlwe_encrypt_zero(const fheacc_params &p, const Tables &T, Rng &r,
                              const uint64_t *sk_ntt, uint64_t *out)
{
    int N = p.N;
    uint64_t *a = out, *b = out + N;
    for (int i = 0; i < N; i++) {
        a[i] = r.uniform(p.Q);
        b[i] = mod_signed(r.gauss(p.E_rlwe), p.Q);
    }
    T.ntt(a);
    T.ntt(b);
    for (int i = 0; i < N; i++) b[i] = addmod(mulmod(a[i], sk_ntt[i], p.Q), b[i], p.Q);
}

static bool params_ok(const fheacc_params *p) { return p && !check_params(*p); }

}  // namespace host
}  // namespace fheacc

using namespace fheacc::host;

extern "C" int fheacc_keygen_lwe_sk(const fheacc_params *p, uint64_t seed, uint64_t *sk)
{
    // LWE_secretkey(RNG_uniform&), LWE.cpp:22-53 (release bounds)
    if (!params_ok(p) || !sk) return FHEACC_EINVAL;
    for (uint64_t attempt = 0;; attempt++) {
        Rng r(seed, TAG_LWE_SK, attempt);
        int64_t s = 0, ss = 0;
        for (int i = 0; i < p->n; i++) {
            int64_t v = r.ternary();
            s += v;
            ss += v < 0 ? -v : v;
            sk[i] = (uint64_t)v % p->q;
        }
        if (!(std::llabs(s) > 200 || ss > 700)) return FHEACC_OK;
        if (attempt > 100000) return FHEACC_EINVAL;
    }
}

extern "C" int fheacc_keygen_rlwe_sk(const fheacc_params *p, uint64_t seed, uint64_t *sk_ntt)
{
    // RLWE_secretkey(RNG_uniform&), RLWE.cpp:243-279 (release bounds)
    if (!params_ok(p) || !sk_ntt) return FHEACC_EINVAL;
    for (uint64_t attempt = 0;; attempt++) {
        Rng r(seed, TAG_RLWE_SK, attempt);
        int64_t s = 0, ss = 0;
        for (int i = 0; i < p->N; i++) {
            int64_t v = r.ternary();
            s += v;
            ss += v < 0 ? -v : v;
            sk_ntt[i] = mod_signed(v, p->Q);
        }
        if (!(std::llabs(s) > 200 || ss > 1300)) break;
        if (attempt > 1000000) return FHEACC_EINVAL;
    }
    Tables T;
    T.build(*p);
    T.ntt(sk_ntt);
    return FHEACC_OK;
}

extern "C" int fheacc_keygen_bootstrap_key(const fheacc_params *p, uint64_t seed, const uint64_t *lwe_sk,
                                           const uint64_t *rlwe_sk_ntt, uint64_t *btkey, int threads)
{
    // bootstrap_key (RLWE.cpp:579-606) of RGSW_ciphertext (RLWE.cpp:561-577)
    // of RGSW_plaintext(value) (RLWE.cpp:512-526).
    if (!params_ok(p) || !lwe_sk || !rlwe_sk_ntt || !btkey) return FHEACC_EINVAL;
    Tables T;
    T.build(*p);
    const int N = p->N, n = p->n;
    const uint64_t q = p->q, Q = p->Q, dG = p->digitG, dR = p->digitR;
    const size_t rw = (size_t)dG * 4 * N;
    std::vector<uint64_t> powbr(dR);
    uint64_t pb = 1;
    for (uint64_t j = 0; j < dR; j++) { powbr[j] = pb; pb = (pb * p->Br) % q; }
    const size_t total = (size_t)p->Br * dR * n;
    parallel_for(total, threads, [&](size_t idx) {
        uint64_t r = idx / (dR * n), j = (idx / n) % dR, k = idx % n;
        uint64_t value = (((r * powbr[j]) % q) * lwe_sk[k]) % q;
        uint64_t mm = value * (2ULL * N / q), sign = 1;
        if (mm >= (uint64_t)N) { mm -= N; sign = Q - 1; }
        std::vector<uint64_t> m(N, 0);
        m[mm] = sign;
        T.ntt(m.data());
        uint64_t *g = btkey + idx * rw;
        uint64_t BG = 1ULL << p->BG_bits;
        for (uint64_t h = 0; h < dG; h++) {
            for (int row = 0; row < 2; row++) {
                uint64_t *c = g + (h * 2 + row) * 2 * (size_t)N;
                Rng rng(seed, TAG_BTKEY, (idx * dG + h) * 2 + row);
                rlwe_encrypt_zero(*p, T, rng, rlwe_sk_ntt, c);
                uint64_t *dst = row == 0 ? c : c + N;  // add_to_a / add_to_b
                for (int i = 0; i < N; i++) dst[i] = addmod(dst[i], m[i], Q);
            }
            for (int i = 0; i < N; i++) m[i] = mulmod(m[i], BG % Q, Q);  // mult_constant_number(BG)
        }
    });
    return FHEACC_OK;
}

extern "C" int fheacc_keygen_lwe_ks_key(const fheacc_params *p, uint64_t seed, const uint64_t *rlwe_sk_ntt,
                                        const uint64_t *lwe_sk, uint64_t *kskey, int threads)
{
    // LWE::keyswitch_key, LWE.cpp:55-106
    if (!params_ok(p) || !lwe_sk || !rlwe_sk_ntt || !kskey) return FHEACC_EINVAL;
    Tables T;
    T.build(*p);
    const int N = p->N, n = p->n;
    const uint64_t q = p->q, Q = p->Q;
    std::vector<uint64_t> z(rlwe_sk_ntt, rlwe_sk_ntt + N);
    T.intt(z.data());
    std::vector<uint64_t> sQ(n);
    for (int i = 0; i < n; i++) sQ[i] = lwe_sk[i] >= q / 2 ? lwe_sk[i] + (Q - q) : lwe_sk[i];
    std::vector<uint64_t> powks(p->digitKS);
    uint64_t pk = 1;
    for (uint32_t j = 0; j < p->digitKS; j++) { powks[j] = pk; pk = mulmod(pk, p->Bks, Q); }
    const size_t total = (size_t)p->Bks * p->digitKS * N;
    parallel_for(total, threads, [&](size_t idx) {
        uint64_t d = idx / ((size_t)p->digitKS * N), j = (idx / N) % p->digitKS, k = idx % N;
        uint64_t mult = mulmod(mulmod(d, powks[j], Q), z[k], Q);
        Rng rng(seed, TAG_LWE_KS, idx);
        uint64_t *c = kskey + idx * ((size_t)n + 1);
        uint64_t b = mod_signed(rng.gauss(p->E_rlwe), Q);
        b = addmod(b, mult, Q);
        for (int h = 0; h < n; h++) {
            c[h] = rng.uniform(Q);
            b = addmod(b, mulmod(c[h], sQ[h], Q), Q);
        }
        c[n] = b;
    });
    return FHEACC_OK;
}

extern "C" int fheacc_keygen_subs_key(const fheacc_params *p, uint64_t seed, const uint64_t *rlwe_sk_ntt,
                                      uint64_t *subs_key, int threads)
{
    // application::substitute_key (app.cpp:4-24) of RLWE::keyswitch_key
    // (RLWE.cpp:293-322), with poly_substitute (RLWE.cpp:23-37).
    if (!params_ok(p) || !rlwe_sk_ntt || !subs_key) return FHEACC_EINVAL;
    Tables T;
    T.build(*p);
    const int N = p->N;
    const uint64_t Q = p->Q, L = p->digitKS_R;
    int logN = T.logN;
    std::vector<uint64_t> s(rlwe_sk_ntt, rlwe_sk_ntt + N);
    T.intt(s.data());
    const size_t total = (size_t)logN * L;
    parallel_for(total, threads, [&](size_t idx) {
        int l = (int)(idx / L);
        uint64_t i = idx % L;
        std::vector<uint64_t> old(N, 0);
        int32_t power = (N >> l) + 1;
        for (int32_t x = 0; x < N; x++) {
            int32_t xo = (x * power) % N;
            old[xo] = ((x * power / N) % 2) == 1 ? (Q - s[x]) % Q : s[x];
        }
        T.ntt(old.data());
        uint64_t f = 1;   // Bks_R^i
        for (uint64_t k = 0; k < i; k++) f = mulmod(f, 1ULL << p->Bks_R_bits, Q);
        Rng rng(seed, TAG_SUBS, idx);
        uint64_t *c = subs_key + idx * 2 * (size_t)N;
        rlwe_encrypt_zero(*p, T, rng, rlwe_sk_ntt, c);
        for (int x = 0; x < N; x++) c[N + x] = addmod(c[N + x], mulmod(old[x], f, Q), Q);
    });
    return FHEACC_OK;
}

extern "C" int fheacc_lwe_encrypt(const fheacc_params *p, uint64_t seed, const uint64_t *lwe_sk,
                                  const uint8_t *bits, size_t count, uint64_t *out)
{
    // LWE_encrypt (LWE.cpp:134-145, release form), plaintext modulus t = 4
    if (!params_ok(p) || !lwe_sk || (!bits && count) || (!out && count)) return FHEACC_EINVAL;
    const int n = p->n;
    const uint64_t q = p->q;
    for (size_t c = 0; c < count; c++) {
        Rng r(seed, TAG_LWE_ENC, c);
        uint64_t *ct = out + c * ((size_t)n + 1);
        uint64_t b = (uint64_t)(r.gauss(p->E) + (int64_t)((uint64_t)(bits[c] & 1) * (q / 4))) % q;
        for (int i = 0; i < n; i++) {
            ct[i] = r.uniform(q);
            b = (b + (ct[i] * lwe_sk[i]) % q) % q;
        }
        ct[n] = b;
    }
    return FHEACC_OK;
}

extern "C" int fheacc_lwe_decrypt(const fheacc_params *p, const uint64_t *lwe_sk, const uint64_t *ct,
                                  size_t count, uint8_t *out)
{
    // LWE_decrypt (LWE.cpp:167-188), t = 4, E = q/16
    if (!params_ok(p) || !lwe_sk || (!ct && count) || (!out && count)) return FHEACC_EINVAL;
    const int n = p->n;
    const uint64_t q = p->q;
    for (size_t c = 0; c < count; c++) {
        const uint64_t *x = ct + c * ((size_t)n + 1);
        uint64_t m = x[n];
        for (int i = 0; i < n; i++) m = (m - x[i] * lwe_sk[i]) % q;
        m = (m + p->E * 2) % q;
        out[c] = (uint8_t)(m * 4 / q);
    }
    return FHEACC_OK;
}

extern "C" int fheacc_rlwe_encrypt(const fheacc_params *p, uint64_t seed, const uint64_t *rlwe_sk_ntt,
                                   const uint64_t *msg_ntt, uint64_t *out)
{
    if (!params_ok(p) || !rlwe_sk_ntt || !msg_ntt || !out) return FHEACC_EINVAL;
    Tables T;
    T.build(*p);
    Rng r(seed, TAG_RLWE_ENC, 0);
    rlwe_encrypt_zero(*p, T, r, rlwe_sk_ntt, out);
    for (int i = 0; i < p->N; i++) out[p->N + i] = addmod(out[p->N + i], msg_ntt[i] % p->Q, p->Q);
    return FHEACC_OK;
}

extern "C" int fheacc_rgsw_encrypt(const fheacc_params *p, uint64_t seed, const uint64_t *rlwe_sk_ntt,
                                   const uint64_t *msg_ntt, uint64_t *out)
{
    // RGSW_ciphertext(m, z) (RLWE.cpp:561-577): row h holds two encryptions of
    // zero, with m * BG^h added to a (c_text[h][0]) and to b (c_text[h][1]).
    if (!params_ok(p) || !rlwe_sk_ntt || !msg_ntt || !out) return FHEACC_EINVAL;
    Tables T;
    T.build(*p);
    const int N = p->N;
    const uint64_t Q = p->Q, BG = (1ULL << p->BG_bits) % Q;
    std::vector<uint64_t> m(N);
    for (int i = 0; i < N; i++) m[i] = msg_ntt[i] % Q;
    for (uint64_t h = 0; h < p->digitG; h++) {
        for (int row = 0; row < 2; row++) {
            uint64_t *c = out + (h * 2 + row) * 2 * (size_t)N;
            Rng rng(seed, TAG_RGSW_ENC, h * 2 + row);
            rlwe_encrypt_zero(*p, T, rng, rlwe_sk_ntt, c);
            uint64_t *dst = row == 0 ? c : c + N;
            for (int i = 0; i < N; i++) dst[i] = addmod(dst[i], m[i], Q);
        }
        for (int i = 0; i < N; i++) m[i] = mulmod(m[i], BG, Q);
    }
    return FHEACC_OK;
}

extern "C" int fheacc_rlwe_phase(const fheacc_params *p, const uint64_t *rlwe_sk_ntt, const uint64_t *ct,
                                 uint64_t *phase_time)
{
    if (!params_ok(p) || !rlwe_sk_ntt || !ct || !phase_time) return FHEACC_EINVAL;
    Tables T;
    T.build(*p);
    const int N = p->N;
    for (int i = 0; i < N; i++)
        phase_time[i] = submod(ct[N + i], mulmod(ct[i], rlwe_sk_ntt[i], p->Q), p->Q);
    T.intt(phase_time);
    return FHEACC_OK;
}
