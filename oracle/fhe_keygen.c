/*
 * fhe_keygen.c -- CPU restatement of the reference's key generation and LWE
 * encryption, part of liboracle.so. TEST INFRASTRUCTURE: it lets the CPU
 * reference arm of bench.py and the tests make keys and ciphertexts without
 * loading the product library.
 *
 * The reference draws from std::default_random_engine seeded by
 * std::random_device (src/RNG.cpp:3-36); here each object draws from its own
 * SplitMix64 stream keyed by (seed, object kind, object index), so the words
 * are reproducible and independent of the thread count. The distributions are
 * the reference's: RNG_uniform(range) uniform on [-range/2, range/2]
 * (src/RNG.cpp:3-17), RNG_norm::generate_norm a normal variate truncated
 * toward zero and reduced '% bound' (src/RNG.cpp:19-36; sigma 3.19 as in the
 * apps). These keys are NOT the product's (its generator differs); they are
 * valid keys of the same parameter set, which is all a timing baseline needs.
 */
#include "fhe_oracle.h"
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;

typedef struct {
    uint64_t s;
} kg_rng;

static uint64_t kg_next(kg_rng *r)
{
    uint64_t z = (r->s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

static kg_rng kg_stream(uint64_t seed, uint64_t kind, uint64_t index)
{
    kg_rng r = {seed * 0xD1B54A32D192ED03ULL ^ (kind << 56) ^ index};
    kg_next(&r);
    return r;
}

/* uniform integer in [0, m) (rejection of the top remainder) */
static uint64_t kg_below(kg_rng *r, uint64_t m)
{
    const uint64_t lim = UINT64_MAX - UINT64_MAX % m;
    for (;;) {
        const uint64_t x = kg_next(r);
        if (x < lim) return x % m;
    }
}

/* RNG_norm::generate_norm(bound) with mean 0, sigma 3.19 (src/RNG.cpp:27-36) */
static int64_t kg_norm(kg_rng *r, uint64_t bound)
{
    const double u1 = ((double)(kg_next(r) >> 11) + 1.0) * 0x1.0p-53;
    const double u2 = (double)(kg_next(r) >> 11) * 0x1.0p-53;
    const double g = 3.19 * sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
    return (int64_t)g % (int64_t)bound;
}

static uint64_t kg_mod(int64_t v, uint64_t m)
{
    const int64_t r = v % (int64_t)m;
    return (uint64_t)(r < 0 ? r + (int64_t)m : r);
}

static uint64_t mulm(uint64_t a, uint64_t b, uint64_t m) { return (uint64_t)((u128)a * b % m); }
static uint64_t addm(uint64_t a, uint64_t b, uint64_t m) { return (uint64_t)(((u128)a + b) % m); }

enum { KG_LWE_SK = 1, KG_RLWE_SK, KG_BTKEY, KG_LWE_KS, KG_LWE_ENC };

/* LWE_secretkey(RNG_uniform(3)) (LWE.cpp:22-53): ternary, redrawn until
 * |sum| <= 200 and sum |s_i| <= 700; stored mod q. */
int ora_keygen_lwe_sk(const ora_params *p, uint64_t seed, uint64_t *sk)
{
    for (uint64_t attempt = 0; attempt < 100000; attempt++) {
        kg_rng r = kg_stream(seed, KG_LWE_SK, attempt);
        int64_t s = 0, ss = 0;
        for (int i = 0; i < p->n; i++) {
            const int64_t v = (int64_t)kg_below(&r, 3) - 1;
            s += v;
            ss += v < 0 ? -v : v;
            sk[i] = kg_mod(v, p->q);
        }
        if (!(llabs(s) > 200 || ss > 700)) return 0;
    }
    return -1;
}

/* RLWE_secretkey(RNG_uniform(3)) (RLWE.cpp:243-279): ternary a, redrawn until
 * |sum| <= 200 and sum |s_i| <= 1300; returned in the NTT domain. */
int ora_keygen_rlwe_sk(const ora_params *p, uint64_t seed, uint64_t *sk_ntt)
{
    for (uint64_t attempt = 0; attempt < 1000000; attempt++) {
        kg_rng r = kg_stream(seed, KG_RLWE_SK, attempt);
        int64_t s = 0, ss = 0;
        for (int i = 0; i < p->N; i++) {
            const int64_t v = (int64_t)kg_below(&r, 3) - 1;
            s += v;
            ss += v < 0 ? -v : v;
            sk_ntt[i] = kg_mod(v, p->Q);
        }
        if (!(llabs(s) > 200 || ss > 1300)) {
            ora_ntt(sk_ntt, p->N, p->Q, p->rou);
            return 0;
        }
    }
    return -1;
}

/* RLWE_encrypt of the zero plaintext (RLWE.cpp:324-344): a uniform and e
 * normal (bound E_rlwe) in the time domain, both transformed, b = a s + e. */
static void kg_rlwe_zero(const ora_params *p, kg_rng *r, const uint64_t *sk_ntt, uint64_t E_rlwe, uint64_t *out)
{
    const int N = p->N;
    uint64_t *a = out, *b = out + N;
    for (int i = 0; i < N; i++) {
        a[i] = kg_below(r, p->Q);
        b[i] = kg_mod(kg_norm(r, E_rlwe), p->Q);
    }
    ora_ntt(a, N, p->Q, p->rou);
    ora_ntt(b, N, p->Q, p->rou);
    for (int i = 0; i < N; i++) b[i] = addm(mulm(a[i], sk_ntt[i], p->Q), b[i], p->Q);
}

typedef struct {
    const ora_params *p;
    uint64_t seed, E_rlwe;
    const uint64_t *lwe_sk, *rlwe_sk_ntt, *z_time;
    uint64_t *out;
    size_t total;
    size_t next;
    pthread_mutex_t mu;
    int kind;
} kg_job;

/* btkey[r][j][k] = RGSW(X^((r Br^j s_k mod q) 2N/q)) (RLWE.cpp:579-606), each
 * RGSW_ciphertext as RLWE.cpp:561-577: row h = two encryptions of zero with
 * m BG^h added to a, then to b; m = RGSW_plaintext (RLWE.cpp:512-526). */
static void kg_btkey_one(kg_job *J, size_t idx, uint64_t *m)
{
    const ora_params *p = J->p;
    const int N = p->N, n = p->n;
    const uint64_t q = p->q, Q = p->Q, dG = p->digitG, dR = p->digitR;
    const uint64_t r = idx / (dR * n), j = (idx / n) % dR, k = idx % n;
    uint64_t powbr = 1;
    for (uint64_t t = 0; t < j; t++) powbr = powbr * p->Br % q;
    const uint64_t value = (r * powbr % q) * J->lwe_sk[k] % q;
    uint64_t mm = value * (2 * (uint64_t)N / q), sign = 1;
    if (mm >= (uint64_t)N) {
        mm -= N;
        sign = Q - 1;
    }
    memset(m, 0, N * sizeof(uint64_t));
    m[mm] = sign;
    ora_ntt(m, N, Q, p->rou);
    uint64_t *g = J->out + idx * dG * 4 * (size_t)N;
    for (uint64_t h = 0; h < dG; h++) {
        for (int row = 0; row < 2; row++) {
            uint64_t *c = g + (h * 2 + row) * 2 * (size_t)N;
            kg_rng rng = kg_stream(J->seed, KG_BTKEY, (idx * dG + h) * 2 + row);
            kg_rlwe_zero(p, &rng, J->rlwe_sk_ntt, J->E_rlwe, c);
            uint64_t *dst = row == 0 ? c : c + N;
            for (int i = 0; i < N; i++) dst[i] = addm(dst[i], m[i], Q);
        }
        const uint64_t BG = ((uint64_t)1 << p->BGbits) % Q;
        for (int i = 0; i < N; i++) m[i] = mulm(m[i], BG, Q);
    }
}

/* kskey[d][j][k] = LWE_Q of d Bks^j z_k under the LWE key moved to mod Q
 * (LWE.cpp:55-106). */
static void kg_ks_one(kg_job *J, size_t idx)
{
    const ora_params *p = J->p;
    const int N = p->N, n = p->n;
    const uint64_t q = p->q, Q = p->Q;
    const uint64_t d = idx / (p->digitKS * (size_t)N), j = (idx / N) % p->digitKS, k = idx % N;
    uint64_t powks = 1;
    for (uint64_t t = 0; t < j; t++) powks = mulm(powks, p->Bks, Q);
    const uint64_t mult = mulm(mulm(d, powks, Q), J->z_time[k], Q);
    kg_rng rng = kg_stream(J->seed, KG_LWE_KS, idx);
    uint64_t *c = J->out + idx * ((size_t)n + 1);
    uint64_t b = addm(kg_mod(kg_norm(&rng, J->E_rlwe), Q), mult, Q);
    for (int h = 0; h < n; h++) {
        const uint64_t s = J->lwe_sk[h] >= q / 2 ? J->lwe_sk[h] + (Q - q) : J->lwe_sk[h];
        c[h] = kg_below(&rng, Q);
        b = addm(b, mulm(c[h], s, Q), Q);
    }
    c[n] = b;
}

static void *kg_worker(void *arg)
{
    kg_job *J = (kg_job *)arg;
    uint64_t *m = (uint64_t *)malloc((size_t)J->p->N * sizeof(uint64_t));
    for (;;) {
        pthread_mutex_lock(&J->mu);
        const size_t idx = J->next++;
        pthread_mutex_unlock(&J->mu);
        if (idx >= J->total) break;
        if (J->kind == KG_BTKEY) kg_btkey_one(J, idx, m);
        else kg_ks_one(J, idx);
    }
    free(m);
    return NULL;
}

static void kg_run(kg_job *J, int threads)
{
    if (threads < 1) threads = 1;
    pthread_mutex_init(&J->mu, NULL);
    J->next = 0;
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * threads);
    for (int t = 1; t < threads; t++) pthread_create(&th[t], NULL, kg_worker, J);
    kg_worker(J);
    for (int t = 1; t < threads; t++) pthread_join(th[t], NULL);
    free(th);
    pthread_mutex_destroy(&J->mu);
}

/* Bootstrap key, layout [Br][digitR][n][digitG][2][2][N]. */
int ora_keygen_bootstrap_key(const ora_params *p, uint64_t seed, uint64_t E_rlwe, const uint64_t *lwe_sk,
                             const uint64_t *rlwe_sk_ntt, uint64_t *btkey, int threads)
{
    kg_job J;
    memset(&J, 0, sizeof J);
    J.p = p; J.seed = seed; J.E_rlwe = E_rlwe; J.lwe_sk = lwe_sk; J.rlwe_sk_ntt = rlwe_sk_ntt; J.out = btkey;
    J.total = (size_t)p->Br * p->digitR * p->n;
    J.kind = KG_BTKEY;
    kg_run(&J, threads);
    return 0;
}

/* LWE key-switch key, layout [Bks][digitKS][N][n+1]. */
int ora_keygen_lwe_ks_key(const ora_params *p, uint64_t seed, uint64_t E_rlwe, const uint64_t *rlwe_sk_ntt,
                          const uint64_t *lwe_sk, uint64_t *kskey, int threads)
{
    uint64_t *z = (uint64_t *)malloc((size_t)p->N * sizeof(uint64_t));
    memcpy(z, rlwe_sk_ntt, (size_t)p->N * sizeof(uint64_t));
    ora_intt(z, p->N, p->Q, p->irou, p->iN);   /* old_key.to_time_domain() */
    kg_job J;
    memset(&J, 0, sizeof J);
    J.p = p; J.seed = seed; J.E_rlwe = E_rlwe; J.lwe_sk = lwe_sk; J.z_time = z; J.out = kskey;
    J.total = (size_t)p->Bks * p->digitKS * p->N;
    J.kind = KG_LWE_KS;
    kg_run(&J, threads);
    free(z);
    return 0;
}

/* LWE_encrypt (LWE.cpp:134-145) of bits with t = 4: b = e + m q/4 + <a, s>
 * mod q, e = generate_norm(E). out: [count][n+1]. */
int ora_lwe_encrypt(const ora_params *p, uint64_t seed, uint64_t E, const uint64_t *sk, const uint8_t *bits,
                    size_t count, uint64_t *out)
{
    const int n = p->n;
    const uint64_t q = p->q;
    for (size_t c = 0; c < count; c++) {
        kg_rng r = kg_stream(seed, KG_LWE_ENC, c);
        uint64_t *ct = out + c * ((size_t)n + 1);
        uint64_t b = kg_mod(kg_norm(&r, E) + (int64_t)((uint64_t)(bits[c] & 1) * (q / 4)), q);
        for (int i = 0; i < n; i++) {
            ct[i] = kg_below(&r, q);
            b = (b + ct[i] * sk[i] % q) % q;
        }
        ct[n] = b;
    }
    return 0;
}
