/*
 * fhe_oracle.c -- CPU restatement of the reference's gate-bootstrapping path.
 *
 * TEST INFRASTRUCTURE: only tests/, __graft_entry__.smoke() and
 * bench.py's CPU baseline / reference arm load this file's library. Nothing in
 * the shipped library links it.
 *
 * Each function names the reference function it restates (file:line, relative
 * to the reference project root FHE_ACC_runtime/). The modular arithmetic keeps
 * the reference's form (a 128-bit product followed by '%', signed differences
 * folded back into [0, Q)), so results are canonical and bit-identical to the
 * reference's, and so is the order of every operation that is not exact.
 *
 * Pinning: tests/test_oracle_golden.py checks this file against the
 * reference's golden transcripts (RLWExRGSW_output.txt, RLWESUBS_output.txt,
 * param_{1k,2k}.txt, committed as fixtures under tests/golden/) and, where the
 * reference was compiled here (oracle/_ref), against the reference itself.
 */
#include "fhe_oracle.h"
#include <stdlib.h>
#include <string.h>
#include <pthread.h>
#include <unistd.h>

typedef unsigned __int128 u128;
typedef __int128 s128;

/* mod_general overloads, nbt.h:59-101 */
static inline uint64_t mod_s128(s128 a, uint64_t m) { return (uint64_t)(((a % (s128)m) + (s128)m) % (s128)m); }
static inline uint64_t mod_u128(u128 a, uint64_t m) { return (uint64_t)(a % (u128)m); }
static inline uint64_t mod_s64(int64_t a, uint64_t m) { return (uint64_t)(((a % (int64_t)m) + (int64_t)m) % (int64_t)m); }

/* ---------------------------------------------------------------- number theory */

uint64_t ora_power_mod(uint64_t base, uint64_t exp, uint64_t mod) /* nbt.cpp:28-47 */
{
    uint64_t b = base % mod;
    u128 r = 1;
    while (exp > 0) {
        if (exp & 1) r = (r * b) % mod;
        b = (uint64_t)(((u128)b * b) % mod);
        exp >>= 1;
    }
    return (uint64_t)r;
}

uint64_t ora_reverse_bit(uint64_t order, uint64_t x) /* nbt.cpp:7-26 */
{
    int bits = 0;
    while ((1ULL << bits) < order) bits++;
    uint64_t r = 0;
    for (int i = 0; i < bits; i++) r |= ((x >> i) & 1ULL) << (bits - 1 - i);
    return r;
}

int ora_is_prime(uint64_t x)
{
    /* The reference uses 20 rounds of Miller-Rabin with random witnesses
     * (nbt.cpp:173-207); the first 12 primes as witnesses decide every
     * 64-bit input exactly. */
    static const uint64_t wit[12] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
    if (x < 2) return 0;
    for (int i = 0; i < 12; i++) {
        if (x == wit[i]) return 1;
        if (x % wit[i] == 0) return 0;
    }
    uint64_t d = x - 1; int s = 0;
    while ((d & 1) == 0) { d >>= 1; s++; }
    for (int i = 0; i < 12; i++) {
        uint64_t y = ora_power_mod(wit[i], d, x);
        if (y == 1 || y == x - 1) continue;
        int comp = 1;
        for (int r = 1; r < s; r++) {
            y = (uint64_t)(((u128)y * y) % x);
            if (y == x - 1) { comp = 0; break; }
        }
        if (comp) return 0;
    }
    return 1;
}

uint64_t ora_find_Q(int nbit, int N) /* nbt.cpp:209-266 via fhe_wo_fpga.cpp:89 */
{
    uint64_t m = 2ULL * (uint64_t)N;
    uint64_t cand = 1ULL << nbit;
    cand = cand + m - (cand % m) + 1;          /* first_prime: Q = 1 mod 2N above 2^nbit */
    while (!ora_is_prime(cand)) cand += m;
    cand -= m;                                  /* previous_prime */
    while (!ora_is_prime(cand)) cand -= m;
    return cand;
}

uint64_t ora_root_of_unity(int N, uint64_t Q) /* nbt.cpp:300-346 */
{
    /* Any primitive 2N-th root w gives all of them as w^k, k odd; the
     * reference returns the smallest (its random generator search only picks
     * the starting root). */
    uint64_t m = 2ULL * (uint64_t)N;
    if ((Q - 1) % m != 0) return 0;
    uint64_t w = 0;
    for (uint64_t x = 2; x < Q; x++) {
        uint64_t c = ora_power_mod(x, (Q - 1) / m, Q);
        if (ora_power_mod(c, (uint64_t)N, Q) == Q - 1) { w = c; break; }
    }
    if (w == 0) return 0;
    uint64_t best = w, w2 = (uint64_t)(((u128)w * w) % Q), cur = w;
    for (uint64_t k = 3; k < m; k += 2) {
        cur = (uint64_t)(((u128)cur * w2) % Q);
        if (cur < best) best = cur;
    }
    return best;
}

static uint64_t *ora_alloc(size_t words) { return (uint64_t *)calloc(words ? words : 1, sizeof(uint64_t)); }

/* --------------------------------------------------------------------- NTT */

void ora_ntt(uint64_t *a, int N, uint64_t Q, const uint64_t *rou) /* nbt.cpp:423-454 */
{
    int t = N;
    for (int m = 1; m < N; m *= 2) {
        t = t / 2;
        for (int i = 0; i < m; i++) {
            int j1 = 2 * i * t, j2 = j1 + t;
            uint64_t S = rou[m + i];
            for (int j = j1; j < j2; j++) {
                uint64_t U = a[j];
                uint64_t V = mod_u128((u128)a[j + t] * (u128)S, Q);
                a[j] = mod_u128((u128)U + (u128)V, Q);
                a[j + t] = mod_s128((s128)U - (s128)V, Q);
            }
        }
    }
}

void ora_intt(uint64_t *a, int N, uint64_t Q, const uint64_t *irou, uint64_t iN) /* nbt.cpp:456-491 */
{
    int t = 1;
    for (int m = N / 2; m >= 1; m /= 2) {
        int j1 = 0;
        for (int i = 0; i < m; i++) {
            int j2 = j1 + t;
            uint64_t S = irou[m + i];
            for (int j = j1; j < j2; j++) {
                uint64_t U = a[j], V = a[j + t];
                a[j] = mod_u128((u128)U + (u128)V, Q);
                a[j + t] = mod_s128(((s128)U - (s128)V) * (s128)S, Q);
            }
            j1 += 2 * t;
        }
        t *= 2;
    }
    for (int i = 0; i < N; i++) a[i] = mod_u128((u128)a[i] * (u128)iN, Q);
}

int ora_params_setup(ora_params *p) /* params.cpp:149-210, fhe_wo_fpga.cpp:95-113 */
{
    int N = p->N;
    if (N < 2 || (N & (N - 1)) || p->Q < 3) return -1;
    p->digitN = 0;
    while ((1 << p->digitN) < N) p->digitN++;
    p->iN = ora_power_mod((uint64_t)N, p->Q - 2, p->Q);
    if (p->ROU == 0) p->ROU = ora_root_of_unity(N, p->Q);
    if (p->ROU == 0) return -1;
    p->rou = ora_alloc((size_t)N);
    p->irou = ora_alloc((size_t)N);
    uint64_t iROU = ora_power_mod(p->ROU, p->Q - 2, p->Q);
    p->rou[0] = 1; p->irou[0] = 1;
    uint64_t t = 1, it = 1;
    for (uint64_t i = 1; i < (uint64_t)N; i++) {
        t = mod_u128((u128)t * p->ROU, p->Q);
        it = mod_u128((u128)it * iROU, p->Q);
        uint64_t r = ora_reverse_bit((uint64_t)N, i);
        p->rou[r] = t;
        p->irou[r] = it;
    }
    /* rotate_vector_gen(false): NTT(-X^(N - 2^j)), params.cpp:196-207 */
    p->rot_bwd = ora_alloc((size_t)p->digitN * (size_t)N);
    int pow2 = 1;
    for (int j = 0; j < p->digitN; j++) {
        uint64_t *v = p->rot_bwd + (size_t)j * N;
        v[N - pow2] = p->Q - 1;
        ora_ntt(v, N, p->Q, p->rou);
        pow2 *= 2;
    }
    /* rotate_vector_gen(true): NTT(X^(2^j)), params.cpp:183-194 (j < log2 N,
       where 2^j < N; the reference's fixed count of 11 fits N = 2048) */
    p->rot_fwd = ora_alloc((size_t)p->digitN * (size_t)N);
    pow2 = 1;
    for (int j = 0; j < p->digitN; j++) {
        uint64_t *v = p->rot_fwd + (size_t)j * N;
        v[pow2] = 1;
        ora_ntt(v, N, p->Q, p->rou);
        pow2 *= 2;
    }
    return 0;
}

void ora_params_free(ora_params *p)
{
    free(p->rou); free(p->irou); free(p->rot_bwd); free(p->rot_fwd);
    p->rou = p->irou = p->rot_bwd = p->rot_fwd = NULL;
}

/* ------------------------------------------------------------ RLWE helpers */

static void rlwe_to_time(const ora_params *p, uint64_t *c) /* RLWE.cpp:188-194 */
{
    ora_intt(c, p->N, p->Q, p->irou, p->iN);
    ora_intt(c + p->N, p->N, p->Q, p->irou, p->iN);
}

static void rlwe_to_freq(const ora_params *p, uint64_t *c) /* RLWE.cpp:180-186 */
{
    ora_ntt(c, p->N, p->Q, p->rou);
    ora_ntt(c + p->N, p->N, p->Q, p->rou);
}

void ora_digit_decompose(const ora_params *p, const uint64_t *rlwe, uint64_t len,
                         uint64_t mask, uint64_t bits, uint64_t *out) /* RLWE.cpp:623-640 */
{
    int N = p->N;
    uint64_t *c = ora_alloc(2 * (size_t)N);
    memcpy(c, rlwe, 2 * (size_t)N * sizeof(uint64_t));
    rlwe_to_time(p, c);
    for (int i = 0; i < N; i++) {
        for (uint64_t j = 0; j < len; j++) {
            out[(j * 2 + 0) * N + i] = c[i] & mask;
            c[i] >>= bits;
            out[(j * 2 + 1) * N + i] = c[N + i] & mask;
            c[N + i] >>= bits;
        }
    }
    for (uint64_t j = 0; j < len; j++) rlwe_to_freq(p, out + j * 2 * N);
    free(c);
}

/* RLWE_mult_NTT_poly + RLWE_addition, RLWE.cpp:432-442 and 377-387:
 * tmp = c1 (.) poly + tmp */
static void rlwe_mac_poly(const ora_params *p, const uint64_t *c1, const uint64_t *poly, uint64_t *tmp)
{
    int N = p->N;
    for (int k = 0; k < N; k++) {
        uint64_t ma = mod_u128((u128)c1[k] * (u128)poly[k], p->Q);
        uint64_t mb = mod_u128((u128)c1[N + k] * (u128)poly[k], p->Q);
        tmp[k] = (ma + tmp[k]) % p->Q;
        tmp[N + k] = (mb + tmp[N + k]) % p->Q;
    }
}

void ora_rlwe_mult_rgsw(const ora_params *p, const uint64_t *acc, const uint64_t *rgsw,
                        uint64_t *out) /* RLWE.cpp:642-704 */
{
    int N = p->N;
    uint64_t dG = p->digitG;
    uint64_t *dec = ora_alloc(dG * 2 * (size_t)N);
    ora_digit_decompose(p, acc, dG, (1ULL << p->BGbits) - 1, p->BGbits, dec);
    uint64_t *tmp = ora_alloc(2 * (size_t)N);
    for (uint64_t i = 0; i < dG; i++) {
        const uint64_t *row0 = rgsw + (i * 2 + 0) * 2 * (size_t)N;   /* c_text[i][0] */
        const uint64_t *row1 = rgsw + (i * 2 + 1) * 2 * (size_t)N;   /* c_text[i][1] */
        rlwe_mac_poly(p, row0, dec + (i * 2 + 0) * (size_t)N, tmp);  /* * decomp[i].a */
        rlwe_mac_poly(p, row1, dec + (i * 2 + 1) * (size_t)N, tmp);  /* * decomp[i].b */
    }
    memcpy(out, tmp, 2 * (size_t)N * sizeof(uint64_t));
    free(tmp); free(dec);
}

void ora_acc_initialization(const ora_params *p, uint64_t embed, uint64_t bound1,
                            uint64_t bound2, uint64_t value, uint64_t *out) /* RLWE.cpp:706-724 */
{
    int N = p->N;
    uint64_t Q8 = p->Q / 8 + 1, negQ8 = p->Q - Q8;
    uint64_t q2 = p->q / 2;
    memset(out, 0, 2 * (size_t)N * sizeof(uint64_t));
    uint64_t *b = out + N;
    for (uint64_t i = 0; i < q2; i++) {
        uint64_t tmp = (uint64_t)((int64_t)value - (int64_t)i) % p->q;  /* mod_pow2, nbt.h:49 */
        if (bound1 < bound2)
            b[i * embed] = ((tmp >= bound1) && (tmp < bound2)) ? negQ8 : Q8;
        else
            b[i * embed] = ((tmp >= bound2) && (tmp < bound1)) ? Q8 : negQ8;
    }
    rlwe_to_freq(p, out);
}

/* ------------------------------------------------------------------- LWE */

void ora_lwe_evaluate(const ora_params *p, const uint64_t *c1, const uint64_t *c2, int gate,
                      uint64_t *out) /* LWE.cpp:203-222 */
{
    int n = p->n;
    uint64_t q = p->q;
    if (gate == 4 || gate == 5) { /* XOR, XNOR */
        out[n] = (2 * (c1[n] - c2[n])) % q;
        for (int i = 0; i < n; i++) out[i] = (2 * (c1[i] - c2[i])) % q;
    } else {
        out[n] = (c1[n] + c2[n]) % q;
        for (int i = 0; i < n; i++) out[i] = (c1[i] + c2[i]) % q;
    }
}

void ora_lwe_eval_not(const ora_params *p, const uint64_t *c, uint64_t *out) /* LWE.cpp:224-231 */
{
    int n = p->n;
    for (int i = 0; i < n; i++) out[i] = (p->q - c[i]) % p->q;
    out[n] = ((p->q / 4) - c[n]) % p->q;
}

static size_t rgsw_words(const ora_params *p) { return (size_t)p->digitG * 4 * (size_t)p->N; }

int ora_blind_rotate(const ora_params *p, const uint64_t *c1, const uint64_t *c2, int gate,
                     const uint64_t *btkey, int fpga_compat, uint64_t *acc_out) /* RLWE.cpp:733-767 */
{
    int n = p->n, N = p->N;
    uint64_t q = p->q;
    uint64_t *c = ora_alloc((size_t)n + 1);
    ora_lwe_evaluate(p, c1, c2, gate, c);
    uint64_t qb1 = p->gate_constant[gate] % q;
    uint64_t qb2 = (qb1 + q / 2) % q;
    uint64_t emb = 2ULL * (uint64_t)N / q;
    ora_acc_initialization(p, emb, qb1, qb2, c[n], acc_out);
    size_t rw = rgsw_words(p);
    uint64_t *tmp = ora_alloc(2 * (size_t)N);
    int steps = 0;
    for (int i = 0; i < n; i++) {
        uint64_t nega = (q - c[i]) % q;
        for (uint64_t j = 0; j < p->digitR; j++) {
            uint64_t residu = nega % p->Br;
            /* issue order: 0 the CPU path's (residue 0 skipped, RLWE.cpp:759);
             * 1 fpga_eval_bootstrap_x4..x16 (every step, myfpga.cpp:1200-1210);
             * 2 fpga_eval_bootstrap_x1 (step (0, 0) always, as BOOTSTRAP_INIT,
             * residue 0 skipped elsewhere, myfpga.cpp:1037-1046) */
            if (residu > 0 || fpga_compat == 1 || (fpga_compat == 2 && i == 0 && j == 0)) {
                const uint64_t *key = btkey + ((residu * p->digitR + j) * (uint64_t)n + (uint64_t)i) * rw;
                ora_rlwe_mult_rgsw(p, acc_out, key, tmp);
                memcpy(acc_out, tmp, 2 * (size_t)N * sizeof(uint64_t));
                steps++;
            }
            nega /= p->Br;
        }
    }
    free(tmp); free(c);
    return steps;
}

void ora_lwe_keyswitch(const ora_params *p, const uint64_t *rlwe, const uint64_t *kskey,
                       uint64_t *out) /* LWE.cpp:233-253 */
{
    int n = p->n, N = p->N;
    uint64_t Q = p->Q;
    uint64_t *c = ora_alloc(2 * (size_t)N);
    memcpy(c, rlwe, 2 * (size_t)N * sizeof(uint64_t));
    for (int i = 0; i < N / 2; i++) {           /* NTT_a_transpose, RLWE.cpp:218-226 */
        uint64_t t = c[i]; c[i] = c[N - 1 - i]; c[N - 1 - i] = t;
    }
    rlwe_to_time(p, c);
    memset(out, 0, ((size_t)n + 1) * sizeof(uint64_t));
    uint64_t Q8 = Q / 8 + 1;
    out[n] = (c[N] + Q8) % Q;
    for (int i = 0; i < N; i++) {
        uint64_t atmp = c[i];
        for (uint64_t j = 0; j < p->digitKS; j++) {
            uint64_t d = atmp % p->Bks;
            const uint64_t *row = kskey + ((d * p->digitKS + j) * (uint64_t)N + (uint64_t)i) * ((uint64_t)n + 1);
            for (int k = 0; k < n; k++) out[k] = mod_s64((int64_t)out[k] - (int64_t)row[k], Q);
            out[n] = mod_s64((int64_t)out[n] - (int64_t)row[n], Q);
            atmp /= p->Bks;
        }
    }
    free(c);
}

uint64_t ora_scale_round(uint64_t x, uint64_t new_mod, uint64_t old_mod) /* LWE.cpp:255-260 */
{
    return (uint64_t)(((u128)old_mod + 2 * (u128)x * (u128)new_mod) / (2 * (u128)old_mod));
}

void ora_lwe_modswitch(const ora_params *p, const uint64_t *in, uint64_t *out) /* LWE.cpp:262-269 */
{
    for (int i = 0; i <= p->n; i++) out[i] = ora_scale_round(in[i], p->q, p->Q);
}

int ora_eval_bootstrap(const ora_params *p, const uint64_t *c1, const uint64_t *c2, int gate,
                       const uint64_t *btkey, const uint64_t *kskey, int fpga_compat,
                       uint64_t *out) /* RLWE.cpp:726-786 */
{
    int n = p->n;
    if (memcmp(c1, c2, ((size_t)n + 1) * sizeof(uint64_t)) == 0) return -1; /* RLWE.cpp:727-730 */
    uint64_t *acc = ora_alloc(2 * (size_t)p->N);
    uint64_t *lq = ora_alloc((size_t)n + 1);
    ora_blind_rotate(p, c1, c2, gate, btkey, fpga_compat, acc);
    ora_lwe_keyswitch(p, acc, kskey, lq);
    ora_lwe_modswitch(p, lq, out);
    free(lq); free(acc);
    return 0;
}

typedef struct {
    const ora_params *p; const uint64_t *c1, *c2; const int32_t *gates; size_t count;
    const uint64_t *btkey, *kskey; int fpga_compat; uint64_t *out;
    size_t next; int failed; pthread_mutex_t mu;
} batch_job;

static void *batch_worker(void *arg)
{
    batch_job *J = (batch_job *)arg;
    size_t w = (size_t)J->p->n + 1;
    for (;;) {
        pthread_mutex_lock(&J->mu);
        size_t i = J->next++;
        pthread_mutex_unlock(&J->mu);
        if (i >= J->count) break;
        int rc = ora_eval_bootstrap(J->p, J->c1 + i * w, J->c2 + i * w, J->gates[i], J->btkey,
                                    J->kskey, J->fpga_compat, J->out + i * w);
        if (rc) { pthread_mutex_lock(&J->mu); J->failed++; pthread_mutex_unlock(&J->mu); }
    }
    return NULL;
}

int ora_eval_bootstrap_batch(const ora_params *p, const uint64_t *c1, const uint64_t *c2,
                             const int32_t *gates, size_t count, const uint64_t *btkey,
                             const uint64_t *kskey, int fpga_compat, int threads,
                             uint64_t *out)
{
    batch_job J;
    memset(&J, 0, sizeof J);
    J.p = p; J.c1 = c1; J.c2 = c2; J.gates = gates; J.count = count;
    J.btkey = btkey; J.kskey = kskey; J.fpga_compat = fpga_compat; J.out = out;
    pthread_mutex_init(&J.mu, NULL);
    if (threads <= 0) threads = (int)sysconf(_SC_NPROCESSORS_ONLN);
    if (threads < 1) threads = 1;
    if ((size_t)threads > count) threads = count ? (int)count : 1;
    pthread_t *tid = (pthread_t *)calloc((size_t)threads, sizeof(pthread_t));
    for (int t = 0; t < threads; t++) pthread_create(&tid[t], NULL, batch_worker, &J);
    for (int t = 0; t < threads; t++) pthread_join(tid[t], NULL);
    free(tid);
    pthread_mutex_destroy(&J.mu);
    return J.failed;
}

uint64_t ora_lwe_decrypt(const ora_params *p, const uint64_t *sk, const uint64_t *c, uint64_t t) /* LWE.cpp:148-190 */
{
    uint64_t q = p->q, m = c[p->n];
    for (int i = 0; i < p->n; i++) m = (m - c[i] * sk[i]) % q;
    m = (m + (q / 16) * 2) % q;   /* E = q/16 in every reference app */
    return m * t / q;
}

/* ---------------------------------------------------- automorphism and KS */

void ora_poly_substitute(const uint64_t *a, int sub_factor, int N, uint64_t Q, uint64_t *out) /* RLWE.cpp:23-37 */
{
    int32_t power = (N >> sub_factor) + 1;
    for (int32_t i = 0; i < N; i++) {
        int32_t io = (i * power) % (int32_t)N;
        if (((i * power / N) % 2) == 1) out[io] = (Q - a[i]) % Q;
        else out[io] = a[i];
    }
}

void ora_rlwe_substitute(const ora_params *p, const uint64_t *c, int sub_factor, uint64_t *out) /* RLWE.cpp:444-462 */
{
    int N = p->N;
    uint64_t *in = ora_alloc(2 * (size_t)N);
    memcpy(in, c, 2 * (size_t)N * sizeof(uint64_t));
    rlwe_to_time(p, in);
    ora_poly_substitute(in, sub_factor, N, p->Q, out);
    ora_poly_substitute(in + N, sub_factor, N, p->Q, out + N);
    rlwe_to_freq(p, out);
    free(in);
}

void ora_rlwe_keyswitch(const ora_params *p, const uint64_t *c, const uint64_t *ksk,
                        uint64_t *out) /* RLWE.cpp:464-510 */
{
    int N = p->N;
    uint64_t Q = p->Q, L = p->digitKS_R;
    uint64_t *dec = ora_alloc(L * 2 * (size_t)N);
    ora_digit_decompose(p, c, L, (1ULL << p->Bks_R_bits) - 1, p->Bks_R_bits, dec);
    uint64_t *o = ora_alloc(2 * (size_t)N);
    memcpy(o + N, c + N, (size_t)N * sizeof(uint64_t));
    for (uint64_t i = 0; i < L; i++) {
        const uint64_t *k = ksk + i * 2 * (size_t)N;
        const uint64_t *d = dec + (i * 2 + 0) * (size_t)N;   /* decomp[i].a */
        for (int x = 0; x < N; x++) {
            uint64_t ma = mod_u128((u128)k[x] * (u128)d[x], Q);        /* RLWE_mult_NTT_poly */
            uint64_t mb = mod_u128((u128)k[N + x] * (u128)d[x], Q);
            o[x] = mod_s64((int64_t)o[x] - (int64_t)ma, Q);           /* RLWE_subtraction */
            o[N + x] = mod_s64((int64_t)o[N + x] - (int64_t)mb, Q);
        }
    }
    memcpy(out, o, 2 * (size_t)N * sizeof(uint64_t));
    free(o); free(dec);
}

void ora_rlwe_rotate_freq_bwd(const ora_params *p, const uint64_t *c, int j, uint64_t *out) /* RLWE.cpp:411-430 */
{
    int N = p->N;
    const uint64_t *v = p->rot_bwd + (size_t)j * N;
    for (int i = 0; i < N; i++) {
        out[i] = mod_u128((u128)c[i] * v[i], p->Q);
        out[N + i] = mod_u128((u128)c[N + i] * v[i], p->Q);
    }
}

void ora_expand_rlwe(const ora_params *p, const uint64_t *c, const uint64_t *subs_key,
                     uint64_t *out) /* app.cpp:26-76 */
{
    int N = p->N;
    size_t rw = 2 * (size_t)N;
    size_t kw = (size_t)p->digitKS_R * rw;
    uint64_t Q = p->Q;
    uint64_t *s1 = ora_alloc(rw), *s2 = ora_alloc(rw), *tmp = ora_alloc(rw), *df = ora_alloc(rw);
    memcpy(out, c, rw * sizeof(uint64_t));
    int inner = 1;
    for (int i = 0; i < p->digitN; i++) {
        for (int j = 0; j < inner; j++) {
            ora_rlwe_substitute(p, out + (size_t)j * rw, i, s1);
            ora_rlwe_keyswitch(p, s1, subs_key + (size_t)i * kw, s2);
            memcpy(tmp, out + (size_t)j * rw, rw * sizeof(uint64_t));
            for (size_t x = 0; x < rw; x++) {
                out[(size_t)j * rw + x] = (tmp[x] + s2[x]) % Q;        /* RLWE_addition */
                df[x] = mod_s64((int64_t)tmp[x] - (int64_t)s2[x], Q);  /* RLWE_subtraction */
            }
            ora_rlwe_rotate_freq_bwd(p, df, i, out + (size_t)(j + inner) * rw);
        }
        inner *= 2;
    }
    free(s1); free(s2); free(tmp); free(df);
}

/* ------------------------------------------------------------- PSI (CMUX) */

/* RLWE_rotate_freq(c, j, forward) (RLWE.cpp:411-430): times NTT(X^(+-2^j)). */
static void rotate_freq(const ora_params *p, const uint64_t *c, int j, int forward, uint64_t *out)
{
    int N = p->N;
    const uint64_t *v = (forward ? p->rot_fwd : p->rot_bwd) + (size_t)j * N;
    for (int i = 0; i < N; i++) {
        out[i] = mod_u128((u128)c[i] * v[i], p->Q);
        out[N + i] = mod_u128((u128)c[N + i] * v[i], p->Q);
    }
}

void ora_cmux(const ora_params *p, const uint64_t *c0, const uint64_t *c1, const uint64_t *sel,
              uint64_t *out) /* RLWE.cpp:788-793 */
{
    size_t rw = 2 * (size_t)p->N;
    uint64_t *diff = ora_alloc(rw), *mult = ora_alloc(rw);
    for (size_t x = 0; x < rw; x++) diff[x] = mod_s64((int64_t)c1[x] - (int64_t)c0[x], p->Q);  /* RLWE_subtraction */
    ora_rlwe_mult_rgsw(p, diff, sel, mult);
    for (size_t x = 0; x < rw; x++) out[x] = (mult[x] + c0[x]) % p->Q;                        /* RLWE_addition */
    free(diff); free(mult);
}

void ora_rlwe_blind_rotate(const ora_params *p, const uint64_t *c, int forward, const uint64_t *rgsws,
                           uint64_t *out) /* RLWE.cpp:824-838 */
{
    size_t rw = 2 * (size_t)p->N;
    size_t gw = p->digitG * 2 * rw;   /* one RGSW: [digitG][2] RLWEs */
    uint64_t *acc = ora_alloc(rw), *tmp = ora_alloc(rw);
    memcpy(acc, c, rw * sizeof(uint64_t));
    for (int i = 0; i < p->digitN; i++) {
        rotate_freq(p, acc, i, forward, tmp);
        ora_cmux(p, acc, tmp, rgsws + (size_t)i * gw, acc);
    }
    memcpy(out, acc, rw * sizeof(uint64_t));
    free(acc); free(tmp);
}

void ora_homo_expand(const ora_params *p, const uint64_t *packed, const uint64_t *enc_sec,
                     const uint64_t *subs_key, uint64_t *out) /* app.cpp:78-96 */
{
    int N = p->N;
    size_t rw = 2 * (size_t)N, dG = p->digitG;
    uint64_t *unpacked = ora_alloc(dG * (size_t)N * rw);
    for (size_t j = 0; j < dG; j++) ora_expand_rlwe(p, packed + j * rw, subs_key, unpacked + j * (size_t)N * rw);
    for (int i = 0; i < N; i++) {
        for (size_t j = 0; j < dG; j++) {
            const uint64_t *u = unpacked + (j * (size_t)N + (size_t)i) * rw;
            uint64_t *row = out + ((size_t)i * dG + j) * 2 * rw;          /* RGSW i, c_text[j] */
            ora_rlwe_mult_rgsw(p, u, enc_sec, row);                        /* c_text[j][0] */
            memcpy(row + rw, u, rw * sizeof(uint64_t));                    /* c_text[j][1] */
        }
    }
    free(unpacked);
}
