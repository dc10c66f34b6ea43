// ref_shim.cpp -- flat C entry points over the reference's own, unmodified
// C++ runtime (FHE_ACC_runtime/src/{nbt,params,RNG,LWE,RLWE,app}.cpp), built by
// oracle/build_ref.sh into oracle/_ref/libref.so where the reference sources are
// present. TEST INFRASTRUCTURE: the tests use it to pin the C restatement in
// fhe_oracle.c against the reference itself; nothing shipped links it.
//
// The shim only copies flat arrays (layouts as in fhe_oracle.h) into the
// reference's classes, sets the reference's global parameters the way its apps
// do (apps/fhe_wo_fpga.cpp:33-162), and calls the reference functions.
#include "params.h"
#include "nbt.h"
#include "LWE.h"
#include "RLWE.h"
#include "app.h"
#include <cstring>
#include <memory>
#include <vector>

extern "C" {

struct ref_params {
    int n; uint64_t q; int N; uint64_t Q;
    uint64_t BGbits, digitG, Br, digitR, Bks, digitKS, Bks_R_bits, digitKS_R;
    uint64_t gate_constant[6];
    uint64_t iN, ROU;   // outputs
};

static RLWE::bootstrap_key *g_bt = nullptr;
static LWE::keyswitch_key *g_ks = nullptr;
static application::substitute_key *g_subs = nullptr;

// Sets the reference globals (fhe_wo_fpga.cpp:35-161). ROU comes from the
// reference's own root_of_unity (nbt.cpp:300); Q must be given.
int ref_setup(ref_params *p)
{
    n = p->n; t = 4; q = p->q; q2 = q / 2; E = q / 16;
    LWE_sk_range = 3; LWE_mean = 0; LWE_stddev = 3.19;
    N = p->N; N2 = N / 2 + 1; digitN = (uint16_t)std::log2((double)N);
    RLWE_sk_range = 3; RLWE_mean = 0; RLWE_stddev = 3.19; E_rlwe = 18; t_rlwe = 8;
    Q = p->Q;
    iN = inverse_mod(N, Q);
    ROU = root_of_unity(N, Q);
    if (ROU_table) free(ROU_table);
    if (iROU_table) free(iROU_table);
    ROU_table = (ciphertext_t *)malloc(N * sizeof(ciphertext_t));
    iROU_table = (ciphertext_t *)malloc(N * sizeof(ciphertext_t));
    root_of_unity_table(ROU, Q, N, ROU_table, iROU_table);
    BG = 1ULL << p->BGbits; BGbits = p->BGbits; BG_mask = BG - 1;
    digitG = p->digitG; digitG2 = 2 * digitG;
    Br = p->Br; digitR = p->digitR;
    Bks = p->Bks; digitKS = p->digitKS;
    Bks_R = 1ULL << p->Bks_R_bits; Bks_R_bits = p->Bks_R_bits; digitKS_R = p->digitKS_R;
    Bks_R_mask = Bks_R - 1;
    for (int i = 0; i < 6; i++) gate_constant[i] = p->gate_constant[i];
    rotate_poly_forward = rotate_vector_gen(true);
    rotate_poly_backward = rotate_vector_gen(false);
    p->iN = iN; p->ROU = ROU;
    return 0;
}

uint64_t ref_find_Q(int nbit, int order) { return previous_prime(first_prime(nbit, order), order); }

void ref_ntt(uint64_t *a) { NTT(a, N, Q, ROU_table); }
void ref_intt(uint64_t *a) { iNTT(a, N, Q, iROU_table, iN); }
void ref_tables(uint64_t *rou, uint64_t *irou)
{
    std::memcpy(rou, ROU_table, N * sizeof(uint64_t));
    std::memcpy(irou, iROU_table, N * sizeof(uint64_t));
}

static RLWE::RLWE_ciphertext to_rlwe(const uint64_t *p)
{
    RLWE::RLWE_ciphertext c;
    for (int i = 0; i < N; i++) { c.a[i] = p[i]; c.b[i] = p[N + i]; }
    c.NTT_form = true;
    return c;
}

static void from_rlwe(const RLWE::RLWE_ciphertext &c, uint64_t *p)
{
    for (int i = 0; i < N; i++) { p[i] = c.a[i]; p[N + i] = c.b[i]; }
}

static RLWE::RGSW_ciphertext to_rgsw(const uint64_t *p)
{
    RLWE::RGSW_ciphertext g;
    for (uint64_t h = 0; h < digitG; h++)
        for (int r = 0; r < 2; r++) g.c_text[h][r] = to_rlwe(p + (h * 2 + r) * 2 * (size_t)N);
    return g;
}

static LWE::LWE_ciphertext to_lwe(const uint64_t *p)
{
    LWE::LWE_ciphertext c;
    for (int i = 0; i < n; i++) c.a[i] = p[i];
    c.b = p[n];
    return c;
}

static void from_lwe(const LWE::LWE_ciphertext &c, uint64_t *p)
{
    for (int i = 0; i < n; i++) p[i] = c.a[i];
    p[n] = c.b;
}

void ref_rlwe_mult_rgsw(const uint64_t *acc, const uint64_t *rgsw, uint64_t *out)
{
    from_rlwe(RLWE::RLWE_mult_RGSW(to_rlwe(acc), to_rgsw(rgsw)), out);
}

void ref_acc_initialization(uint64_t embed, uint64_t b1, uint64_t b2, uint64_t value, uint64_t *out)
{
    from_rlwe(RLWE::acc_initialization(embed, b1, b2, value), out);
}

// Loads flat keys (layouts of fhe_oracle.h) into the reference's key classes.
void ref_load_keys(const uint64_t *btkey, const uint64_t *kskey)
{
    delete g_bt; delete g_ks;
    g_bt = new RLWE::bootstrap_key();
    g_ks = new LWE::keyswitch_key();
    size_t rw = (size_t)digitG * 4 * N;
    g_bt->btkey.resize(Br);
    for (uint64_t r = 0; r < Br; r++) {
        g_bt->btkey[r].resize(digitR);
        for (uint64_t j = 0; j < digitR; j++) {
            g_bt->btkey[r][j].resize(n);
            for (int i = 0; i < n; i++)
                g_bt->btkey[r][j][i] = to_rgsw(btkey + ((r * digitR + j) * n + i) * rw);
        }
    }
    g_ks->kskey.resize(Bks);
    for (uint64_t d = 0; d < Bks; d++) {
        g_ks->kskey[d].resize(digitKS);
        for (uint64_t j = 0; j < digitKS; j++) {
            g_ks->kskey[d][j].resize(N);
            for (int i = 0; i < N; i++)
                g_ks->kskey[d][j][i] = to_lwe(kskey + ((d * digitKS + j) * N + i) * (size_t)(n + 1));
        }
    }
}

void ref_free_keys(void)
{
    delete g_bt; delete g_ks; delete g_subs;
    g_bt = nullptr; g_ks = nullptr; g_subs = nullptr;
}

int ref_eval_bootstrap(const uint64_t *c1, const uint64_t *c2, int gate, uint64_t *out)
{
    if (!g_bt || !g_ks) return -1;
    LWE::LWE_ciphertext a = to_lwe(c1), b = to_lwe(c2);
    if (a == b) return -1;   // the reference exits here (RLWE.cpp:727-730)
    from_lwe(RLWE::eval_bootstrap(a, b, *g_bt, *g_ks, (GATES)gate), out);
    return 0;
}

void ref_lwe_keyswitch(const uint64_t *rlwe, uint64_t *out)
{
    from_lwe(LWE::LWE_keyswitch(to_rlwe(rlwe), *g_ks), out);
}

void ref_lwe_modswitch(const uint64_t *in, uint64_t *out)
{
    from_lwe(LWE::LWE_modswitch(to_lwe(in)), out);
}

void ref_rlwe_substitute(const uint64_t *c, int f, uint64_t *out)
{
    from_rlwe(RLWE::RLWE_substitute(to_rlwe(c), f), out);
}

void ref_rlwe_keyswitch(const uint64_t *c, const uint64_t *ksk, uint64_t *out)
{
    RLWE::keyswitch_key k;
    k.RLWE_kskey.resize(digitKS_R);
    for (uint64_t i = 0; i < digitKS_R; i++) k.RLWE_kskey[i] = to_rlwe(ksk + i * 2 * (size_t)N);
    from_rlwe(RLWE::RLWE_keyswitch(to_rlwe(c), k), out);
}

void ref_expand_rlwe(const uint64_t *c, const uint64_t *subs, uint64_t *out)
{
    application::substitute_key sk;
    sk.subs_key.resize(digitN);
    size_t kw = (size_t)digitKS_R * 2 * N;
    for (int l = 0; l < digitN; l++) {
        sk.subs_key[l].RLWE_kskey.resize(digitKS_R);
        for (uint64_t i = 0; i < digitKS_R; i++)
            sk.subs_key[l].RLWE_kskey[i] = to_rlwe(subs + l * kw + i * 2 * (size_t)N);
    }
    auto r = application::expand_RLWE(to_rlwe(c), sk);
    for (int i = 0; i < N; i++) from_rlwe((*r)[i], out + (size_t)i * 2 * N);
}

static application::substitute_key to_subs(const uint64_t *subs)
{
    application::substitute_key sk;
    sk.subs_key.resize(digitN);
    size_t kw = (size_t)digitKS_R * 2 * N;
    for (int l = 0; l < digitN; l++) {
        sk.subs_key[l].RLWE_kskey.resize(digitKS_R);
        for (uint64_t i = 0; i < digitKS_R; i++)
            sk.subs_key[l].RLWE_kskey[i] = to_rlwe(subs + l * kw + i * 2 * (size_t)N);
    }
    return sk;
}

void ref_cmux(const uint64_t *c0, const uint64_t *c1, const uint64_t *sel, uint64_t *out)
{
    from_rlwe(RLWE::CMUX(to_rlwe(c0), to_rlwe(c1), to_rgsw(sel)), out);
}

// blind_rotate (RLWE.cpp:824-838) takes exactly num_rotate_poly RGSWs (a
// constant 11 in params.h) and exits otherwise; returns -1 without calling it.
int ref_blind_rotate(const uint64_t *c, int forward, const uint64_t *rgsws, int count, uint64_t *out)
{
    if (count != (int)num_rotate_poly) return -1;
    std::vector<RLWE::RGSW_ciphertext> C;
    const size_t gw = digitG * 4 * (size_t)N;
    for (int i = 0; i < count; i++) C.push_back(to_rgsw(rgsws + i * gw));
    from_rlwe(RLWE::blind_rotate(to_rlwe(c), forward != 0, C), out);
    return 0;
}

void ref_homo_expand(const uint64_t *packed, const uint64_t *enc_sec, const uint64_t *subs, uint64_t *out)
{
    auto bits = std::make_unique<std::vector<RLWE::RLWE_ciphertext>>(digitG);
    for (uint64_t j = 0; j < digitG; j++) (*bits)[j] = to_rlwe(packed + j * 2 * (size_t)N);
    auto r = application::homo_expand(bits, to_rgsw(enc_sec), to_subs(subs));
    const size_t gw = digitG * 4 * (size_t)N;
    for (int i = 0; i < N; i++)
        for (uint64_t h = 0; h < digitG; h++)
            for (int g = 0; g < 2; g++) from_rlwe((*r)[i].c_text[h][g], out + i * gw + (h * 2 + g) * 2 * (size_t)N);
}

}  // extern "C"
