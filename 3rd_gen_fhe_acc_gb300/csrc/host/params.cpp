// params.cpp -- parameter presets, derivation and twiddle tables.
// Replaces the per-app global setup of the reference runtime
// (apps/fhe_wo_fpga.cpp:33-162, params.cpp:149-210, nbt.cpp:209-346).
#include "host_math.hpp"
#include <cstring>

namespace fheacc {
namespace host {

uint64_t powmod(uint64_t b, uint64_t e, uint64_t m)
{
    uint64_t r = 1 % m;
    b %= m;
    while (e) {
        if (e & 1) r = mulmod(r, b, m);
        b = mulmod(b, b, m);
        e >>= 1;
    }
    return r;
}

bool is_prime(uint64_t x)
{
    // Deterministic Miller-Rabin; the first 12 prime witnesses decide every
    // 64-bit input (the reference draws 20 random witnesses, nbt.cpp:173).
    static const uint64_t wit[12] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
    if (x < 2) return false;
    for (uint64_t w : wit) {
        if (x == w) return true;
        if (x % w == 0) return false;
    }
    uint64_t d = x - 1;
    int s = 0;
    while (!(d & 1)) { d >>= 1; s++; }
    for (uint64_t w : wit) {
        uint64_t y = powmod(w, d, x);
        if (y == 1 || y == x - 1) continue;
        bool comp = true;
        for (int r = 1; r < s && comp; r++) {
            y = mulmod(y, y, x);
            if (y == x - 1) comp = false;
        }
        if (comp) return false;
    }
    return true;
}

uint64_t reverse_bits(uint64_t x, int bits)
{
    uint64_t r = 0;
    for (int i = 0; i < bits; i++) r |= ((x >> i) & 1ULL) << (bits - 1 - i);
    return r;
}

static uint64_t shoup_companion(uint64_t w, uint64_t Q) { return (uint64_t)(((u128)w << 64) / Q); }

// x * w mod Q, with ws = shoup_companion(w); result canonical.
static inline uint64_t shoup_mul(uint64_t x, uint64_t w, uint64_t ws, uint64_t Q)
{
    uint64_t t = (uint64_t)(((u128)x * ws) >> 64);
    uint64_t r = x * w - t * Q;
    return r >= Q ? r - Q : r;
}

void Tables::build(const fheacc_params &p)
{
    N = p.N;
    logN = 0;
    while ((1 << logN) < N) logN++;
    Q = p.Q;
    iN = p.iN;
    rou.assign(N, 0); irou.assign(N, 0); rou_s.assign(N, 0); irou_s.assign(N, 0);
    uint64_t iROU = powmod(p.ROU, Q - 2, Q);
    rou[0] = 1; irou[0] = 1;
    uint64_t t = 1, it = 1;
    for (int i = 1; i < N; i++) {
        t = mulmod(t, p.ROU, Q);
        it = mulmod(it, iROU, Q);
        uint64_t r = reverse_bits((uint64_t)i, logN);
        rou[r] = t;
        irou[r] = it;
    }
    for (int i = 0; i < N; i++) {
        rou_s[i] = shoup_companion(rou[i], Q);
        irou_s[i] = shoup_companion(irou[i], Q);
    }
    iN_s = shoup_companion(iN, Q);
}

void Tables::ntt(uint64_t *a) const
{
    int t = N;
    for (int m = 1; m < N; m *= 2) {
        t >>= 1;
        for (int i = 0; i < m; i++) {
            uint64_t w = rou[m + i], ws = rou_s[m + i];
            uint64_t *x = a + 2 * i * t, *y = x + t;
            for (int j = 0; j < t; j++) {
                uint64_t u = x[j], v = shoup_mul(y[j], w, ws, Q);
                x[j] = addmod(u, v, Q);
                y[j] = submod(u, v, Q);
            }
        }
    }
}

void Tables::intt(uint64_t *a) const
{
    int t = 1;
    for (int m = N / 2; m >= 1; m /= 2) {
        for (int i = 0; i < m; i++) {
            uint64_t w = irou[m + i], ws = irou_s[m + i];
            uint64_t *x = a + 2 * i * t, *y = x + t;
            for (int j = 0; j < t; j++) {
                uint64_t u = x[j], v = y[j];
                x[j] = addmod(u, v, Q);
                y[j] = shoup_mul(submod(u, v, Q), w, ws, Q);
            }
        }
        t <<= 1;
    }
    for (int i = 0; i < N; i++) a[i] = shoup_mul(a[i], iN, iN_s, Q);
}

static int ceil_log(uint64_t base, uint64_t x)
{
    // smallest d with base^d >= x: ceil(log(x) / log(base)) for x not a power
    // of base, as the apps compute digit counts (fhe_wo_fpga.cpp:122-138).
    int d = 0;
    u128 v = 1;
    while (v < x) { v *= base; d++; }
    return d;
}

const char *check_params(const fheacc_params &p)
{
    if (p.N != 1024 && p.N != 2048 && p.N != 512 && p.N != 256) return "N must be 256, 512, 1024 or 2048";
    if (p.q < 4 || (p.q & (p.q - 1))) return "q must be a power of two >= 4";
    if ((2u * (uint32_t)p.N) % p.q) return "q must divide 2N";
    if (p.n < 1 || p.n > 4096) return "n out of range";
    if (p.Q < 3 || p.Q >= (1ULL << 62)) return "Q must be in [3, 2^62)";
    if ((p.Q - 1) % (2ULL * (uint64_t)p.N)) return "Q must be 1 mod 2N";
    if (!is_prime(p.Q)) return "Q must be prime";
    if (p.BG_bits < 1 || p.BG_bits > 30 || p.digitG < 1) return "bad gadget base";
    if ((uint64_t)p.BG_bits * p.digitG < 64 && (1ULL << (p.BG_bits * p.digitG)) < p.Q) return "digitG too small for Q";
    if (p.Br < 2 || p.digitR < 1) return "bad refresh base";
    if (p.Bks < 2 || p.digitKS < 1) return "bad key-switch base";
    if (p.Bks_R_bits < 1 || p.Bks_R_bits > 30 || p.digitKS_R < 1) return "bad RLWE key-switch base";
    if (p.ROU == 0 || p.iN == 0) return "parameters not derived";
    return nullptr;
}

}  // namespace host
}  // namespace fheacc

using namespace fheacc::host;

extern "C" int fheacc_params_preset(int preset, fheacc_params *out)
{
    if (!out) return FHEACC_EINVAL;
    std::memset(out, 0, sizeof *out);
    out->q = 512;
    out->Br = 23;
    out->Bks = 25;
    out->Bks_R_bits = 9;
    out->E_rlwe = 18;
    switch (preset) {
    case 0: out->n = 500; out->N = 1024; out->nbit = 27; out->BG_bits = 7; break;
    case 1: out->n = 630; out->N = 2048; out->nbit = 54; out->BG_bits = 9; break;
    case 2: out->n = 512; out->N = 1024; out->nbit = 27; out->BG_bits = 9; break;
    default: return FHEACC_EINVAL;
    }
    return fheacc_params_derive(out);
}

extern "C" int fheacc_params_derive(fheacc_params *p)
{
    if (!p || p->N < 2 || (p->N & (p->N - 1)) || p->q < 2) return FHEACC_EINVAL;
    uint64_t m = 2ULL * (uint64_t)p->N;
    if (p->Q == 0) {
        if (p->nbit < 12 || p->nbit > 61) return FHEACC_EINVAL;
        // Q = previous_prime(first_prime(nbit, N), N), nbt.cpp:209-266
        uint64_t c = 1ULL << p->nbit;
        c = c + m - (c % m) + 1;
        while (!is_prime(c)) c += m;
        c -= m;
        while (!is_prime(c)) c -= m;
        p->Q = c;
    }
    if (p->BG_bits == 0 || p->Br < 2 || p->Bks < 2 || p->Bks_R_bits == 0) return FHEACC_EINVAL;
    if (p->digitG == 0) p->digitG = (uint32_t)ceil_log(1ULL << p->BG_bits, p->Q);
    if (p->digitR == 0) p->digitR = (uint32_t)ceil_log(p->Br, p->q);
    if (p->digitKS == 0) p->digitKS = (uint32_t)ceil_log(p->Bks, p->Q);
    if (p->digitKS_R == 0) p->digitKS_R = (uint32_t)ceil_log(1ULL << p->Bks_R_bits, p->Q);
    bool gz = true;
    for (int i = 0; i < 6; i++) gz = gz && p->gate_constant[i] == 0;
    if (gz) {
        uint64_t q8 = p->q >> 3;   // fhe_wo_fpga.cpp:141-146
        p->gate_constant[0] = 5 * q8;  // OR
        p->gate_constant[1] = 7 * q8;  // AND
        p->gate_constant[2] = 1 * q8;  // NOR
        p->gate_constant[3] = 3 * q8;  // NAND
        p->gate_constant[4] = 5 * q8;  // XOR
        p->gate_constant[5] = 1 * q8;  // XNOR
    }
    if ((p->Q - 1) % m) return FHEACC_EINVAL;
    p->iN = powmod((uint64_t)p->N % p->Q, p->Q - 2, p->Q);
    if (p->ROU == 0) {
        // smallest primitive 2N-th root of unity (nbt.cpp:300-346)
        uint64_t w = 0;
        for (uint64_t x = 2; x < p->Q && !w; x++) {
            uint64_t c = powmod(x, (p->Q - 1) / m, p->Q);
            if (powmod(c, (uint64_t)p->N, p->Q) == p->Q - 1) w = c;
        }
        if (!w) return FHEACC_EINVAL;
        uint64_t best = w, w2 = mulmod(w, w, p->Q), cur = w;
        for (uint64_t k = 3; k < m; k += 2) {
            cur = mulmod(cur, w2, p->Q);
            if (cur < best) best = cur;
        }
        p->ROU = best;
    }
    if (p->E == 0) p->E = p->q / 16;
    if (p->E_rlwe == 0) p->E_rlwe = 18;
    return check_params(*p) ? FHEACC_EINVAL : FHEACC_OK;
}

extern "C" size_t fheacc_bootstrap_key_words(const fheacc_params *p)
{
    if (!p) return 0;
    return (size_t)p->Br * p->digitR * (size_t)p->n * p->digitG * 4 * (size_t)p->N;
}

extern "C" size_t fheacc_lwe_ks_key_words(const fheacc_params *p)
{
    if (!p) return 0;
    return (size_t)p->Bks * p->digitKS * (size_t)p->N * ((size_t)p->n + 1);
}

extern "C" size_t fheacc_subs_key_words(const fheacc_params *p)
{
    if (!p) return 0;
    int logN = 0;
    while ((1 << logN) < p->N) logN++;
    return (size_t)logN * p->digitKS_R * 2 * (size_t)p->N;
}

extern "C" int fheacc_twiddle_tables(const fheacc_params *p, uint64_t *rou, uint64_t *irou)
{
    if (!p || !rou || !irou || check_params(*p)) return FHEACC_EINVAL;
    Tables t;
    t.build(*p);
    std::memcpy(rou, t.rou.data(), (size_t)p->N * 8);
    std::memcpy(irou, t.irou.data(), (size_t)p->N * 8);
    return FHEACC_OK;
}
