/*
 * fhe_oracle.h -- CPU restatement of the FHEW/AP gate-bootstrapping path of
 * zhehongw/3rd_Gen_FHE_ACC (FHE_ACC_runtime), used ONLY as test infrastructure.
 *
 * TEST INFRASTRUCTURE. Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference arm of bench.py may load this library. The product
 * (libfheacc.so, libfheacc_host.so and the Python package) never links or
 * calls it.
 *
 * Every function restates one reference function; the reference file:line
 * it follows is given beside each declaration (paths are relative to the
 * reference project root). Arithmetic deliberately keeps the reference's
 * style (unsigned __int128 products followed by '%'), so that the restatement
 * is easy to audit line by line against the reference.
 *
 * Data layouts (all words are uint64_t, the reference's ciphertext_t):
 *   poly            : N words. NTT-domain polys are in the reference's
 *                     bit-reversed order (nbt.cpp:423-454).
 *   RLWE            : a[N] then b[N]                      (RLWE.h:127-159)
 *   RGSW            : [digitG][2 rows g][2 polys a,b][N]  (RLWE.h:313-329,
 *                     c_text[h][g].a / .b)
 *   bootstrap key   : [Br][digitR][n] RGSW                 (RLWE.h:331-345)
 *   LWE             : a[n] then b                           (LWE.h:36-64)
 *   LWE ks key      : [Bks][digitKS][N] LWE (n+1 words)     (LWE.h:86-101)
 *   RLWE ks key     : [digitKS_R] RLWE                      (RLWE.h:181-195)
 *   substitute key  : [digitN] RLWE ks key                  (app.h:22-28)
 */
#ifndef FHE_ORACLE_H
#define FHE_ORACLE_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Parameter set; mirrors the reference's global parameters (params.h:11-134). */
typedef struct ora_params {
    int      n;          /* LWE dimension                                  */
    uint64_t q;          /* LWE modulus, power of two                      */
    int      N;          /* ring dimension, power of two                   */
    uint64_t Q;          /* RLWE prime modulus, Q = 1 mod 2N               */
    uint64_t BGbits;     /* gadget base 2^BGbits                           */
    uint64_t digitG;     /* gadget digits                                  */
    uint64_t Br;         /* refresh base                                   */
    uint64_t digitR;     /* refresh digits                                 */
    uint64_t Bks;        /* RLWE->LWE key switch base                      */
    uint64_t digitKS;    /* RLWE->LWE key switch digits                    */
    uint64_t Bks_R_bits; /* RLWE->RLWE key switch base 2^Bks_R_bits        */
    uint64_t digitKS_R;  /* RLWE->RLWE key switch digits                   */
    uint64_t gate_constant[6];
    /* derived by ora_params_setup */
    uint64_t iN;         /* N^-1 mod Q                                     */
    uint64_t ROU;        /* smallest primitive 2N-th root of unity mod Q   */
    uint64_t *rou;       /* N words, psi^bitrev(i)                         */
    uint64_t *irou;      /* N words, psi^-bitrev(i)                        */
    int      digitN;     /* log2 N                                         */
    uint64_t *rot_bwd;   /* [digitN][N]: NTT(-X^(N-2^j))  (params.cpp:177) */
    uint64_t *rot_fwd;   /* [digitN][N]: NTT(X^(2^j))     (params.cpp:183) */
} ora_params;

/* Miller-Rabin with a fixed witness set (exact for 64-bit inputs); stands in
 * for the randomised MR_primality (nbt.cpp:173-207). */
int      ora_is_prime(uint64_t x);
/* Q = previous_prime(first_prime(nbit, N), N) as the reference apps compute
 * it (fhe_wo_fpga.cpp:89; nbt.cpp:209-266). */
uint64_t ora_find_Q(int nbit, int N);
/* smallest primitive 2N-th root of unity (nbt.cpp:300-346). */
uint64_t ora_root_of_unity(int N, uint64_t Q);
uint64_t ora_power_mod(uint64_t base, uint64_t exp, uint64_t mod);   /* nbt.cpp:28  */
uint64_t ora_reverse_bit(uint64_t order, uint64_t x);                /* nbt.cpp:7   */

/* Fill derived fields (iN, ROU, tables); params.cpp:149-210,
 * fhe_wo_fpga.cpp:95-113. Returns 0 on success. */
int  ora_params_setup(ora_params *p);
void ora_params_free(ora_params *p);

/* in-place negacyclic CT NTT, bit-reversed output   (nbt.cpp:423-454) */
void ora_ntt(uint64_t *a, int N, uint64_t Q, const uint64_t *rou);
/* in-place GS inverse NTT with *N^-1                   (nbt.cpp:456-491) */
void ora_intt(uint64_t *a, int N, uint64_t Q, const uint64_t *irou, uint64_t iN);

/* digit_decompose (RLWE.cpp:623-640): out = [len][2][N], NTT domain. */
void ora_digit_decompose(const ora_params *p, const uint64_t *rlwe, uint64_t len,
                         uint64_t mask, uint64_t bits, uint64_t *out);
/* RLWE_mult_RGSW (RLWE.cpp:642-704). acc and out are NTT-domain RLWEs. */
void ora_rlwe_mult_rgsw(const ora_params *p, const uint64_t *acc, const uint64_t *rgsw,
                        uint64_t *out);
/* acc_initialization (RLWE.cpp:706-724). out is an NTT-domain RLWE. */
void ora_acc_initialization(const ora_params *p, uint64_t embed, uint64_t bound1,
                            uint64_t bound2, uint64_t value, uint64_t *out);
/* LWE_evaluate (LWE.cpp:203-222). */
void ora_lwe_evaluate(const ora_params *p, const uint64_t *c1, const uint64_t *c2, int gate,
                      uint64_t *out);
/* LWE_eval_NOT (LWE.cpp:224-231). */
void ora_lwe_eval_not(const ora_params *p, const uint64_t *c, uint64_t *out);
/* Blind rotation part of eval_bootstrap (RLWE.cpp:733-767): the NTT-domain
 * accumulator after all steps. fpga_compat = 1 also applies the residue-0
 * keys, as fpga_eval_bootstrap_x4..x16 do (myfpga.cpp:1200-1210); 2 applies
 * the first step (i = 0, j = 0) whatever its residue and skips residue 0
 * elsewhere, the issue order of fpga_eval_bootstrap_x1 (myfpga.cpp:1037-1046).
 * Returns the number of RLWE x RGSW steps applied. */
int  ora_blind_rotate(const ora_params *p, const uint64_t *c1, const uint64_t *c2, int gate,
                      const uint64_t *btkey, int fpga_compat, uint64_t *acc_out);
/* LWE_keyswitch (LWE.cpp:233-253): RLWE (NTT) -> LWE mod Q. */
void ora_lwe_keyswitch(const ora_params *p, const uint64_t *rlwe, const uint64_t *kskey,
                       uint64_t *out);
/* scale_round / LWE_modswitch (LWE.cpp:255-269). */
uint64_t ora_scale_round(uint64_t x, uint64_t new_mod, uint64_t old_mod);
void ora_lwe_modswitch(const ora_params *p, const uint64_t *in, uint64_t *out);
/* eval_bootstrap (RLWE.cpp:726-786). Returns 0, or -1 when c1 == c2
 * (where the reference calls exit(1)). */
int  ora_eval_bootstrap(const ora_params *p, const uint64_t *c1, const uint64_t *c2, int gate,
                        const uint64_t *btkey, const uint64_t *kskey, int fpga_compat,
                        uint64_t *out);
/* eval_bootstrap over a batch on `threads` POSIX threads (threads <= 0: all
 * online cores). c1/c2/out are [count][n+1]. Returns the number of failed
 * gates (c1 == c2). */
int  ora_eval_bootstrap_batch(const ora_params *p, const uint64_t *c1, const uint64_t *c2,
                              const int32_t *gates, size_t count, const uint64_t *btkey,
                              const uint64_t *kskey, int fpga_compat, int threads,
                              uint64_t *out);
/* LWE_decrypt (LWE.cpp:148-190), plaintext modulus t. */
uint64_t ora_lwe_decrypt(const ora_params *p, const uint64_t *sk, const uint64_t *c, uint64_t t);

/* poly_substitute (RLWE.cpp:23-37), time domain. */
void ora_poly_substitute(const uint64_t *a, int sub_factor, int N, uint64_t Q, uint64_t *out);
/* RLWE_substitute (RLWE.cpp:444-462): NTT RLWE in, NTT RLWE out. */
void ora_rlwe_substitute(const ora_params *p, const uint64_t *c, int sub_factor, uint64_t *out);
/* RLWE_keyswitch (RLWE.cpp:464-510): NTT RLWE in/out, ksk = [digitKS_R] RLWE. */
void ora_rlwe_keyswitch(const ora_params *p, const uint64_t *c, const uint64_t *ksk,
                        uint64_t *out);
/* RLWE_rotate_freq(c, j, false) (RLWE.cpp:411-430). */
void ora_rlwe_rotate_freq_bwd(const ora_params *p, const uint64_t *c, int j, uint64_t *out);
/* expand_RLWE (app.cpp:26-76): out = [N] NTT RLWEs. */
void ora_expand_rlwe(const ora_params *p, const uint64_t *c, const uint64_t *subs_key,
                     uint64_t *out);

/* CMUX (RLWE.cpp:788-793): RLWE_mult_RGSW(c1 - c0, sel) + c0; NTT RLWEs,
   sel an RGSW [digitG][2][2][N]. */
void ora_cmux(const ora_params *p, const uint64_t *c0, const uint64_t *c1, const uint64_t *sel,
              uint64_t *out);
/* blind_rotate (RLWE.cpp:824-838): log2 N CMUXes with rotations by
   X^(+-2^i); rgsws = [log2 N] RGSWs. out may alias c. */
void ora_rlwe_blind_rotate(const ora_params *p, const uint64_t *c, int forward, const uint64_t *rgsws,
                           uint64_t *out);
/* homo_expand (app.cpp:78-96): digitG packed RLWEs -> N RGSWs
   [N][digitG][2][2][N]; row j of RGSW i = (RLWE_mult_RGSW(u, enc_sec), u),
   u = expand_RLWE(packed[j])[i]. */
void ora_homo_expand(const ora_params *p, const uint64_t *packed, const uint64_t *enc_sec,
                     const uint64_t *subs_key, uint64_t *out);

/* Key generation and LWE encryption (fhe_keygen.c): the reference's key
 * formats and distributions from a seeded generator of the oracle's own (not
 * the product's words). */
int ora_keygen_lwe_sk(const ora_params *p, uint64_t seed, uint64_t *sk);              /* LWE.cpp:22-53   */
int ora_keygen_rlwe_sk(const ora_params *p, uint64_t seed, uint64_t *sk_ntt);         /* RLWE.cpp:243-279 */
int ora_keygen_bootstrap_key(const ora_params *p, uint64_t seed, uint64_t E_rlwe, const uint64_t *lwe_sk,
                             const uint64_t *rlwe_sk_ntt, uint64_t *btkey, int threads);   /* RLWE.cpp:561-606 */
int ora_keygen_lwe_ks_key(const ora_params *p, uint64_t seed, uint64_t E_rlwe, const uint64_t *rlwe_sk_ntt,
                          const uint64_t *lwe_sk, uint64_t *kskey, int threads);         /* LWE.cpp:55-106  */
int ora_lwe_encrypt(const ora_params *p, uint64_t seed, uint64_t E, const uint64_t *sk, const uint8_t *bits,
                    size_t count, uint64_t *out);                                        /* LWE.cpp:134-145 */

#ifdef __cplusplus
}
#endif
#endif
