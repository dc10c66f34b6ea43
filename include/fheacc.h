/*
 * fheacc.h -- C ABI of libfheacc.so, the GB300 (sm_103a) device backend for the
 * FHEW/AP gate-bootstrapping path of zhehongw/3rd_Gen_FHE_ACC.
 *
 * The library replaces the runtime's AWS-F1 device backend (namespace FPGA,
 * FHE_ACC_runtime/include/myfpga.h:128-404). Each entry point below names the
 * reference interface it stands in for. Plain pointers and sizes only; every
 * function returns an int status (FHEACC_OK or a negative FHEACC_E* code) and
 * never exits or aborts. fheacc_last_error() describes the last failure.
 *
 * Word formats follow the reference's ciphertext_t (uint64_t):
 *   LWE   : a[n] then b                  (LWE.h:36-64)            n+1 words
 *   RLWE  : a[N] then b[N], NTT domain in the reference's bit-reversed
 *           order (RLWE.h:127-159, nbt.cpp:423-454)               2N words
 *   RGSW  : [digitG][2 rows][2 polys a,b][N]  = c_text[h][g].a/.b  (RLWE.h:313-329)
 *   bootstrap key : [Br][digitR][n] RGSW  = btkey[r][j][i]        (RLWE.h:331-345)
 *   LWE key-switch key : [Bks][digitKS][N] LWE mod Q = kskey[d][j][i] (LWE.h:86-101)
 *   substitute key : [log2 N][digitKS_R] RLWE = subs_key[l].RLWE_kskey[k] (app.h:22-28)
 *   gates : int32, the reference's enum GATES {OR, AND, NOR, NAND, XOR, XNOR}
 *           (params.h:107)
 */
#ifndef FHEACC_H
#define FHEACC_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FHEACC_OK          0
#define FHEACC_EINVAL    (-22)   /* bad argument / parameter set             */
#define FHEACC_ENOMEM    (-12)   /* host or device allocation failed         */
#define FHEACC_ENODEV    (-19)   /* no usable CUDA device                    */
#define FHEACC_EIO        (-5)   /* CUDA error                               */
#define FHEACC_ETIMEDOUT (-110)  /* fheacc_sync / bounded device wait expired */
#define FHEACC_ENOKEY    (-126)  /* required key not uploaded               */
#define FHEACC_EBUSY     (-16)   /* serving queue full                       */
#define FHEACC_EMISMATCH (-74)   /* device key differs from the given key    */

/* flags for the bootstrap calls */
#define FHEACC_FLAG_FPGA_COMPAT 1u  /* also apply residue-0 keys, as
                                       fpga_eval_bootstrap_x4..x16 do
                                       (myfpga.cpp:1200-1210) */
#define FHEACC_FLAG_PROFILE     2u  /* record CUDA events around each kernel of
                                       the call, on the launching stream;
                                       read them with fheacc_kernel_times */
#define FHEACC_FLAG_FPGA_X1     4u  /* the issue order of fpga_eval_bootstrap_x1
                                       (myfpga.cpp:1031-1063): the first step
                                       (i = 0, j = 0) is always applied, with
                                       its residue's key even when the residue
                                       is 0 (BOOTSTRAP_INIT carries the key
                                       address), every later step only with a
                                       non-zero residue. FHEACC_FLAG_FPGA_COMPAT,
                                       which applies every step, takes
                                       precedence. */

enum fheacc_gate { FHEACC_OR = 0, FHEACC_AND, FHEACC_NOR, FHEACC_NAND, FHEACC_XOR, FHEACC_XNOR };

/* Parameter set. Replaces the reference's mutable globals (params.h:11-134)
 * and the OCL register file pushed by FPGA::OCL_config_wr_rd
 * (myfpga.cpp:82-326). Fields marked (derived) are filled by
 * fheacc_params_derive when zero. */
typedef struct fheacc_params {
    int32_t  n;              /* LWE dimension                          */
    uint32_t q;              /* LWE modulus, power of two              */
    int32_t  N;              /* ring dimension, 1024 or 2048           */
    uint32_t nbit;           /* Q = largest prime < 2^nbit, Q = 1 mod 2N (if Q == 0) */
    uint64_t Q;              /* RLWE modulus                           */
    uint32_t BG_bits;        /* gadget base 2^BG_bits                  */
    uint32_t digitG;         /* (derived) ceil(log_BG Q)               */
    uint32_t Br;             /* refresh base                           */
    uint32_t digitR;         /* (derived) ceil(log_Br q)               */
    uint32_t Bks;            /* RLWE->LWE key-switch base              */
    uint32_t digitKS;        /* (derived) ceil(log_Bks Q)              */
    uint32_t Bks_R_bits;     /* RLWE->RLWE key-switch base 2^Bks_R_bits */
    uint32_t digitKS_R;      /* (derived) ceil(log_Bks_R Q)            */
    uint64_t gate_constant[6]; /* (derived) OR..XNOR bound1, fhe_wo_fpga.cpp:141-146 */
    uint64_t iN;             /* (derived) N^-1 mod Q                   */
    uint64_t ROU;            /* (derived) smallest primitive 2N-th root of unity */
    uint32_t E;              /* (derived) LWE noise bound q/16         */
    uint32_t E_rlwe;         /* RLWE noise bound (reference: 18)       */
} fheacc_params;

/* Presets of the workloads this backend is measured on.
 *  0 : n=500, N=1024, Q=134215681 (largest prime < 2^27, = 1 mod 2N),
 *      BG=2^7 x4 digits, Br=23, Bks=25, Bks_R=2^9, q=512
 *  1 : n=630, N=2048, Q=18014398509404161 (< 2^54), BG=2^9 x6, Br=23,
 *      Bks=25, Bks_R=2^9, q=512
 *  2 : the reference CPU app's set (fhe_wo_fpga.cpp:35-146): n=512, N=1024,
 *      Q=134215681, BG=2^9 x3, Br=23, Bks=25, Bks_R=2^9, q=512 */
int fheacc_params_preset(int preset, fheacc_params *out);
/* Fill the (derived) fields; fhe_wo_fpga.cpp:89-161. */
int fheacc_params_derive(fheacc_params *p);

/* Sizes, in 64-bit words, of the key formats above. */
size_t fheacc_bootstrap_key_words(const fheacc_params *p);
size_t fheacc_lwe_ks_key_words(const fheacc_params *p);
size_t fheacc_subs_key_words(const fheacc_params *p);

/* Twiddle tables (psi^bitrev(i), psi^-bitrev(i)), root_of_unity_table,
 * params.cpp:149-175. rou/irou: N words each. */
int fheacc_twiddle_tables(const fheacc_params *p, uint64_t *rou, uint64_t *irou);

/* ---------------------------------------------------------------- host side
 * Key generation and encryption (host, no GPU). Deterministic from `seed`:
 * the same seed gives the same words on every machine. These keep the
 * reference's key-generation API (LWE.cpp:22-146, RLWE.cpp:243-606,
 * app.cpp:4-24) behind plain arrays. threads <= 0 uses all online cores. */
int fheacc_keygen_lwe_sk(const fheacc_params *p, uint64_t seed, uint64_t *sk /* n */);
int fheacc_keygen_rlwe_sk(const fheacc_params *p, uint64_t seed, uint64_t *sk_ntt /* N */);
int fheacc_keygen_bootstrap_key(const fheacc_params *p, uint64_t seed, const uint64_t *lwe_sk,
                                const uint64_t *rlwe_sk_ntt, uint64_t *btkey, int threads);
int fheacc_keygen_lwe_ks_key(const fheacc_params *p, uint64_t seed, const uint64_t *rlwe_sk_ntt,
                             const uint64_t *lwe_sk, uint64_t *kskey, int threads);
int fheacc_keygen_subs_key(const fheacc_params *p, uint64_t seed, const uint64_t *rlwe_sk_ntt,
                           uint64_t *subs_key, int threads);
/* LWE_encrypt of bits (m * q/4), LWE.cpp:108-146. out: [count][n+1]. */
int fheacc_lwe_encrypt(const fheacc_params *p, uint64_t seed, const uint64_t *lwe_sk,
                       const uint8_t *bits, size_t count, uint64_t *out);
/* LWE_decrypt with t = 4, LWE.cpp:148-190. out: count values in [0, 4). */
int fheacc_lwe_decrypt(const fheacc_params *p, const uint64_t *lwe_sk, const uint64_t *ct,
                       size_t count, uint8_t *out);
/* RLWE_encrypt of an NTT-domain plaintext poly, RLWE.cpp:324-344. */
int fheacc_rlwe_encrypt(const fheacc_params *p, uint64_t seed, const uint64_t *rlwe_sk_ntt,
                        const uint64_t *msg_ntt, uint64_t *out /* 2N */);
/* RGSW_ciphertext(m, z) (RLWE.cpp:561-577): RGSW encryption of the NTT-domain
 * plaintext msg_ntt, reference layout [digitG][2][2][N]. */
int fheacc_rgsw_encrypt(const fheacc_params *p, uint64_t seed, const uint64_t *rlwe_sk_ntt,
                        const uint64_t *msg_ntt, uint64_t *out);
/* b - a*s in NTT domain, then inverse NTT: the noisy time-domain phase
 * (RLWE_decrypt before denoise, RLWE.cpp:346-357). */
int fheacc_rlwe_phase(const fheacc_params *p, const uint64_t *rlwe_sk_ntt, const uint64_t *ct,
                      uint64_t *phase_time /* N */);

/* -------------------------------------------------------------- device side */
typedef struct fheacc_ctx fheacc_ctx;

/* Create a context on CUDA device `device`: derives the parameter set and
 * builds the twiddle tables on the device. Replaces OCL_config_wr_rd
 * (myfpga.cpp:82-326) and BAR1_ROU_table_{1k,2k}_wr (myfpga.cpp:399-594).
 * A context is used by one host thread at a time, and its asynchronous calls
 * on different streams must not overlap: they share the context's scratch
 * (accumulators, staging, claim and window counters), as the reference's
 * FPGA slot is used by one caller at a time. For concurrent work use one
 * context per stream (keys are uploaded to each), or a CUDA graph
 * (fheacc_graph_*), which owns its scratch. */
int fheacc_create(const fheacc_params *p, int device, fheacc_ctx **out);
int fheacc_destroy(fheacc_ctx *ctx);
/* Last error message of ctx (or of the last failed create when ctx is NULL). */
const char *fheacc_last_error(const fheacc_ctx *ctx);
int fheacc_get_params(const fheacc_ctx *ctx, fheacc_params *out);
/* Device memory held by the context (keys, tables, scratch), in bytes. */
size_t fheacc_device_bytes(const fheacc_ctx *ctx);

/* Key upload, host words in the formats above; re-laid-out for the device
 * once, at upload. Replace dma_write_bootstrap_key (myfpga.cpp:596-656),
 * dma_write_subs_key (myfpga.cpp:658-712). The LWE key-switch key has no FPGA
 * counterpart (the FPGA runtime key-switches on the host, myfpga.cpp:1519). */
int fheacc_upload_bootstrap_key(fheacc_ctx *ctx, const uint64_t *btkey, size_t words);
int fheacc_upload_lwe_ks_key(fheacc_ctx *ctx, const uint64_t *kskey, size_t words);
int fheacc_upload_subs_key(fheacc_ctx *ctx, const uint64_t *subs_key, size_t words);

/* Read-back verification of a resident key: FHEACC_OK if the device copy is
 * word for word what uploading `btkey` / `subs_key` (same formats and sizes as
 * the uploads) would make, FHEACC_EMISMATCH at the first step tile (bootstrap
 * key) or key (substitute key) that differs, FHEACC_ENOKEY if none was
 * uploaded. Blocking; temporary device memory of one step tile (64-bit words:
 * the whole substitute key). Replace dma_read_compare_bootstrap_key
 * (myfpga.cpp:772-851) and dma_read_compare_subs_key (myfpga.cpp:853-925). */
int fheacc_verify_bootstrap_key(fheacc_ctx *ctx, const uint64_t *btkey, size_t words);
int fheacc_verify_subs_key(fheacc_ctx *ctx, const uint64_t *subs_key, size_t words);

/* Gate bootstrapping of `count` independent gates, HOST buffers, blocking:
 * out[i] = eval_bootstrap(c1[i], c2[i], gates[i]) (RLWE.cpp:726-786).
 * Replaces fpga_eval_bootstrap_x1/_x4/_x8/_x12/_x16 (myfpga.cpp:1003-1660)
 * with any count. c1/c2/out: [count][n+1]. A gate with c1 == c2 returns
 * FHEACC_EINVAL (the CPU path exits, the FPGA path returns rc = -1). */
int fheacc_bootstrap(fheacc_ctx *ctx, const uint64_t *c1, const uint64_t *c2,
                     const int32_t *gates, size_t count, uint64_t *out, uint32_t flags);
/* Same, DEVICE buffers, asynchronous on `stream` (a cudaStream_t; NULL is the
 * legacy default stream, as in the CUDA runtime). Inputs are not checked for
 * c1 == c2. All *_async calls and the sub-steps below follow the same stream
 * rule; fheacc_sync waits for the most recent of them. */
int fheacc_bootstrap_async(fheacc_ctx *ctx, const uint64_t *d_c1, const uint64_t *d_c2,
                           const int32_t *d_gates, size_t count, uint64_t *d_out,
                           uint32_t flags, void *stream);
/* Gate bootstrapping that allocates nothing, DEVICE buffers, asynchronous on
 * `stream`; same results as fheacc_bootstrap_async. No counterpart in the
 * reference. It is meant for callers that may not allocate while they run:
 * fheacc_bootstrap_async grows the context's scratch with cudaMalloc/cudaFree
 * (cudaFree synchronises the whole device), which a serving loop sharing the
 * GPU with other streams, a process under a fixed device-memory reservation,
 * or a real-time loop cannot accept. Here the scratch is a fixed device array
 * inside the library (776 KiB, present on every GPU that loads it until exit),
 * so at most FHEACC_NOALLOC_MAX_GATES gates per call; larger counts return
 * FHEACC_EINVAL. Parameter sets with N = 1024 only. The first call on a
 * device looks up the array's device address (make that first call before any
 * stream capture). All calls share the one array: calls whose work overlaps on
 * the GPU (different streams, or different contexts on the same device) race
 * and give wrong results; order them on one stream or synchronise. Each call
 * resets the array's claim counter and key-switch partial sums with
 * cudaMemsetAsync on `stream` (no allocation), then launches the kernels;
 * FHEACC_FLAG_PROFILE records the same events as fheacc_bootstrap_async. Keys
 * must have been uploaded to ctx beforehand. */
#define FHEACC_NOALLOC_MAX_GATES 64
int fheacc_bootstrap_noalloc(fheacc_ctx *ctx, const uint64_t *d_c1, const uint64_t *d_c2,
                             const int32_t *d_gates, size_t count, uint64_t *d_out, uint32_t flags,
                             void *stream);

/* The plain form: one launch sequence per gate (the per-gate issue of
 * fpga_eval_bootstrap_x1, myfpga.cpp:1003-1127), DEVICE buffers. */
int fheacc_bootstrap_plain_async(fheacc_ctx *ctx, const uint64_t *d_c1, const uint64_t *d_c2,
                                 const int32_t *d_gates, size_t count, uint64_t *d_out,
                                 uint32_t flags, void *stream);

/* Sub-steps of the path, DEVICE buffers, asynchronous (parity checks).
 * Forward / inverse negacyclic NTT of `count` polys in place
 * (nbt.cpp:423-454 / 456-491). Inputs canonical (< Q); outputs canonical. */
int fheacc_ntt_forward(fheacc_ctx *ctx, uint64_t *d_polys, size_t count, void *stream);
int fheacc_ntt_inverse(fheacc_ctx *ctx, uint64_t *d_polys, size_t count, void *stream);
/* RLWE_mult_RGSW (RLWE.cpp:642-704) of count accumulators, each with its own
 * RGSW (reference layout). */
int fheacc_rlwe_mult_rgsw(fheacc_ctx *ctx, const uint64_t *d_acc, const uint64_t *d_rgsw,
                          uint64_t *d_out, size_t count, void *stream);
/* Blind rotation of eval_bootstrap (RLWE.cpp:733-767): NTT accumulators out,
 * [count][2N]. */
int fheacc_blind_rotate_async(fheacc_ctx *ctx, const uint64_t *d_c1, const uint64_t *d_c2,
                              const int32_t *d_gates, size_t count, uint64_t *d_acc,
                              uint32_t flags, void *stream);
/* LWE_keyswitch (LWE.cpp:233-253): NTT RLWEs -> LWE mod Q, [count][n+1]. */
int fheacc_lwe_keyswitch_async(fheacc_ctx *ctx, const uint64_t *d_rlwe, size_t count,
                               uint64_t *d_out, void *stream);
/* LWE_modswitch (LWE.cpp:262-269): LWE mod Q -> LWE mod q. */
int fheacc_lwe_modswitch_async(fheacc_ctx *ctx, const uint64_t *d_in, size_t count,
                               uint64_t *d_out, void *stream);

/* Launch-shape options of the blind-rotation kernel.
 *  FHEACC_OPT_BR_REGS_FOR_3 : 1 or -1 (default) = the register budget of 3
 *                             resident CTAs per SM, 0 = of 2 CTAs per SM
 *  FHEACC_OPT_BR_CTAS_PER_SM: cap on resident CTAs per SM, 0 = occupancy limit
 *  FHEACC_OPT_BR_GROUP      : cap on the ciphertexts a CTA carries through the
 *                             bootstrap key together (its step-outer group;
 *                             0 = the kernel's maximum, 24 for 32-bit words,
 *                             8 for 64-bit); the launch fits equal groups to
 *                             the batch under the cap
 *  FHEACC_OPT_BR_WINDOW     : 64-bit words: steps per bucket of the step
 *                             window that keeps the CTAs of a launch within
 *                             two buckets of each other, so that the key tiles
 *                             they read stay in L2; 0 = off, -1 (default) = 1
 *  FHEACC_OPT_BR_PIPES      : pipelines (32-bit words) or workers (64-bit)
 *                             per CTA, 1..3; 0 = default: 32-bit 1 up to 2
 *                             gates per SM, 2 up to 5, else 3; 64-bit 1 up to
 *                             1 gate per SM, else 2. The pipelines of a CTA
 *                             share its group of ciphertexts item by item, so
 *                             they finish together; with one per CTA, up to 3
 *                             CTAs share an SM and finish at different times.
 *  FHEACC_OPT_BR_POOL       : 64-bit words: when the batch does not divide
 *                             evenly among the CTAs, each CTA takes
 *                             count / CTAs ciphertexts of its own and all
 *                             CTAs share the remainder step by step; 0 = off
 *                             (some CTAs take one ciphertext more), -1
 *                             (default) = on
 *  FHEACC_OPT_KS_TILED      : LWE key switch of a batched bootstrap:
 *                             1 = the tiled form (gate blocks sharing each
 *                             key row group through shared memory) for any
 *                             batch, 0 = one CTA per gate, -1 (default) =
 *                             tiled from 1024 gates (32-bit words) or from
 *                             two gates per SM (64-bit words)
 *  FHEACC_OPT_BR_SOLO       : 32-bit words: the latency form of the blind
 *                             rotation (one CTA per ciphertext, accumulator in
 *                             shared memory, each step's key prefetched into
 *                             shared memory by bulk asynchronous copies) up
 *                             to this many gates per SM; 0 = off, -1
 *                             (default) = 1. Not taken when
 *                             FHEACC_OPT_BR_PIPES or
 *                             FHEACC_OPT_DEBUG_WAIT_LIMIT is set.
 *  FHEACC_OPT_DEBUG_WAIT_LIMIT: for tests of the error path only. The
 *                             number of polls (64-bit workers, the step
 *                             window) or idle periods (32-bit pipelines) a
 *                             bounded wait may take before it gives up;
 *                             -1 (default) = the built-in limits. With a
 *                             small value the waits between the workers of a
 *                             CTA expire: the kernel still returns, the
 *                             launch's results are invalid,
 *                             FHEACC_STATUS_WAIT_LIMIT is set and
 *                             fheacc_sync / fheacc_bootstrap return
 *                             FHEACC_EIO. Set it back to -1 afterwards.
 * Results never depend on the other options. The 64-bit blind rotation is a
 * cooperative launch whenever its CTAs wait on each other (the remainder
 * pool, the step window), so a grid that cannot be co-resident fails to
 * launch rather than waiting. */
#define FHEACC_OPT_BR_REGS_FOR_3  1
#define FHEACC_OPT_BR_CTAS_PER_SM 2
#define FHEACC_OPT_BR_GROUP       3
#define FHEACC_OPT_BR_WINDOW      4
#define FHEACC_OPT_BR_PIPES       5
#define FHEACC_OPT_BR_POOL        6
#define FHEACC_OPT_DEBUG_WAIT_LIMIT 7
#define FHEACC_OPT_KS_TILED       8
#define FHEACC_OPT_BR_SOLO        9
int fheacc_set_option(fheacc_ctx *ctx, int option, int value);

/* Per-kernel device times (ms) of the most recent call made with
 * FHEACC_FLAG_PROFILE: ms[0] blind rotation, ms[1] key switch + modulus
 * switch. Waits for that call to finish. */
int fheacc_kernel_times(fheacc_ctx *ctx, float ms[2]);
/* Measures this device's 32-bit integer multiply-add throughput (IMAD lane
 * operations per second) with a short dependent-chain kernel of this library;
 * the denominator of the integer roofline. */
int fheacc_measure_imad_rate(fheacc_ctx *ctx, double *imad_per_s);
/* Measures this device's L2 read bandwidth (bytes per second): a streaming
 * read of a buffer of a third of L2, resident after a warm-up sweep, by every
 * SM with 16-byte L2-only loads; the peak against which the blind rotation's
 * key streaming (RGSW words served from L2) is reported. */
int fheacc_measure_l2_read_rate(fheacc_ctx *ctx, double *bytes_per_s);
/* SM time, in ns per unit per SM, of the pieces of one blind-rotation step run
 * alone at the blind-rotation kernel's occupancy: ns[0] forward NTT, ns[1]
 * digit NTT (table-driven first stages), ns[2] inverse NTT, ns[3] multiply-
 * accumulate of one RLWE x RGSW step with keys streamed from L2. 32-bit
 * parameter sets with the bootstrap key uploaded. */
int fheacc_measure_components(fheacc_ctx *ctx, double ns[4]);

/* Picks the blind rotation's launch options (the FHEACC_OPT_BR_* above)
 * for batches of `count` gates: times every candidate on a synthetic batch of
 * that size (uniform LWE inputs mod q, the six gates in turn) with this
 * context's keys, and leaves the fastest set on the context. `trials` (may be
 * NULL) receives up to max_trials of the candidates with their times and
 * *n_trials (may be NULL) their number. Results are unchanged by the options;
 * only the launch shape differs. The reference has no counterpart (the FPGA
 * runtime's in-flight count is a constant, myfpga.cpp:1533). */
typedef struct fheacc_tune_trial {
    int regs_for_3;    /* FHEACC_OPT_BR_REGS_FOR_3 value */
    int ctas_per_sm;   /* FHEACC_OPT_BR_CTAS_PER_SM value */
    int group;         /* FHEACC_OPT_BR_GROUP value */
    int window;        /* FHEACC_OPT_BR_WINDOW value */
    int pipes;         /* FHEACC_OPT_BR_PIPES value */
    float ms;          /* one bootstrap of the synthetic batch, best of two */
} fheacc_tune_trial;
int fheacc_autotune(fheacc_ctx *ctx, size_t count, fheacc_tune_trial *trials, int max_trials, int *n_trials);

/* ------------------------------------------------------------- containers
 * One self-describing file per object (host/container.cpp): a 64-byte header
 * (magic "FHEACC01", kind, parameter-set fingerprint, word count, FNV-1a
 * checksum) and the words in the host layouts above. The reference keeps
 * keys only in memory and regenerates them each run. Loads fail with
 * FHEACC_EINVAL on another kind, parameter set or size, FHEACC_EIO on a short
 * or corrupted file. */
#define FHEACC_KIND_LWE_SK        1u
#define FHEACC_KIND_RLWE_SK       2u
#define FHEACC_KIND_BOOTSTRAP_KEY 3u
#define FHEACC_KIND_LWE_KS_KEY    4u
#define FHEACC_KIND_SUBS_KEY      5u
#define FHEACC_KIND_LWE_CT        6u   /* [count][n+1] */
#define FHEACC_KIND_RLWE_CT       7u   /* [count][2N]  */
#define FHEACC_KIND_RGSW_CT       8u   /* [count][digitG][2][2][N] */
int fheacc_container_save(const char *path, uint32_t kind, const fheacc_params *p, const uint64_t *words,
                          size_t count);
int fheacc_container_load(const char *path, uint32_t kind, const fheacc_params *p, uint64_t *words, size_t count);
int fheacc_container_info(const char *path, uint32_t *kind, uint64_t *fingerprint, size_t *count);

/* -------------------------------------------------------------- PSI (CMUX)
 * The RLWE-level operations of the reference's PSI application. Ciphertexts
 * are canonical NTT-domain RLWEs [2N] (u64); RGSWs in the reference layout
 * [digitG][2][2][N]. */
/* CMUX (RLWE.cpp:788-793) of count pairs: out[i] = RLWE_mult_RGSW(c1[i] -
 * c0[i], sel) + c0[i]. c0[i] / c1[i] sit at d_c0 / d_c1 + i * in_stride words
 * (0: 2N, contiguous; 4N picks the pairs (v[2i], v[2i+1]) of one array for a
 * tree level); out is contiguous and may alias d_c0 when in_stride is 2N. One
 * RGSW per pair, or one for all with sel_shared = 1. */
int fheacc_cmux_async(fheacc_ctx *ctx, const uint64_t *d_c0, const uint64_t *d_c1, size_t in_stride,
                      const uint64_t *d_sel, int sel_shared, uint64_t *d_out, size_t count, void *stream);
/* blind_rotate (RLWE.cpp:824-838) of count RLWEs, each rotated by the
 * private amount that log2 N RGSWs (shared by all) encode: log2 N CMUXes with
 * the NTT-domain rotations by X^(2^i) (forward) or X^(-2^i). (The reference's
 * fixed count of 11, params.h num_rotate_poly, is log2 N for N = 2048.) */
int fheacc_rlwe_blind_rotate_async(fheacc_ctx *ctx, const uint64_t *d_in, const uint64_t *d_rgsws, int forward,
                                   uint64_t *d_out, size_t count, void *stream);
/* homo_expand (app.cpp:78-96): digitG packed RLWEs -> N RGSWs [N][digitG][2][2][N]
 * (row j of RGSW i = (RLWE_mult_RGSW(u, enc_sec), u), u = expand_RLWE(packed
 * [j])[i]); needs the substitute key. */
int fheacc_homo_expand(fheacc_ctx *ctx, const uint64_t *d_packed, const uint64_t *d_enc_sec, uint64_t *d_out,
                       void *stream);

/* ------------------------------------------------------------------- graphs
 * A fixed set of batched gate bootstraps, over one or more contexts (parameter
 * sets, e.g. an N = 1024 and an N = 2048 context) of one device, replayed with
 * one CUDA-graph launch. Batches run in the order they were added; with
 * FHEACC_GRAPH_CONCURRENT each context's batches form their own branch and the
 * branches run concurrently (useful for small batches; large ones finish
 * sooner in order, as each fills the GPU on its own). The graph is
 * captured at the first launch after an add, owns its scratch, and reads the
 * device buffers given to fheacc_graph_add_bootstrap at every launch (they and
 * the contexts must outlive the graph). Outputs equal fheacc_bootstrap_async
 * on the same inputs. No counterpart in the reference, whose runtime holds one
 * parameter set per process (params.h). */
typedef struct fheacc_graph fheacc_graph;
#define FHEACC_GRAPH_CONCURRENT 1u
int fheacc_graph_create(fheacc_graph **out, uint32_t flags);
int fheacc_graph_add_bootstrap(fheacc_graph *g, fheacc_ctx *ctx, const uint64_t *d_c1, const uint64_t *d_c2,
                               const int32_t *d_gates, size_t count, uint64_t *d_out);
/* Enqueues the whole graph on `stream` (NULL: the legacy default stream). */
int fheacc_graph_launch(fheacc_graph *g, void *stream);
size_t fheacc_graph_batches(const fheacc_graph *g);
const char *fheacc_graph_last_error(const fheacc_graph *g);
int fheacc_graph_destroy(fheacc_graph *g);

/* ----------------------------------------------------------------- serving
 * A continuous-batching request loop over the gate bootstrap (no counterpart
 * in the reference, whose FPGA driver runs one fixed-width batch at a time,
 * myfpga.cpp:1130-1660). A request is a gate circuit: num_inputs LWE
 * ciphertexts ([num_inputs][n+1] host words), then num_gates gates; gate g
 * computes node num_inputs + g = eval_bootstrap(node in1[g], node in2[g],
 * gate_types[g]) with in1[g] != in2[g] < num_inputs + g. The last num_outputs
 * nodes are written to `out` ([num_outputs][n+1]) when the request completes.
 * All nodes of an admitted request live in a device pool of pool_ciphertexts
 * slots (0: sized at creation from the device memory then free, a quarter of
 * it up to 32 GiB); a request is admitted when the pool has room for all its
 * nodes, in arrival order, and a request larger than the whole pool is
 * refused with FHEACC_EINVAL. A worker thread keeps up to two rounds in
 * flight on two streams, each with its own scratch: whenever a round ends or
 * a lane is free, every gate of every admitted request whose inputs are ready
 * and that is not already in flight (up to max_batch) goes into one batched
 * launch, so requests arriving while a round runs start on the other lane
 * without waiting for it. Both parameter widths are served (N = 1024 and
 * N = 2048 contexts). Keys must be uploaded before fheacc_server_create; the
 * context must outlive the server and not be used for other work while the
 * server runs. */
typedef struct fheacc_server fheacc_server;
typedef struct fheacc_request_done {
    uint64_t request_id;
    int32_t status;          /* FHEACC_OK or an error code */
    double queue_ms;         /* submission to admission */
    double latency_ms;       /* submission to completion */
} fheacc_request_done;
typedef struct fheacc_server_stats_t {
    uint64_t rounds, gates;  /* batched launches and gates run so far */
    double busy_s;           /* wall time during which at least one round was on the GPU */
    uint64_t waiting, active, free_slots;
    uint64_t pool_slots;     /* ciphertexts the pool holds */
    uint64_t lanes;          /* rounds the server keeps in flight at once */
} fheacc_server_stats_t;
int fheacc_server_create(fheacc_ctx *ctx, size_t max_batch, size_t pool_ciphertexts, fheacc_server **out);
int fheacc_server_submit(fheacc_server *srv, const uint64_t *inputs, uint32_t num_inputs, const int32_t *gate_types,
                         const uint32_t *in1, const uint32_t *in2, uint32_t num_gates, uint32_t num_outputs,
                         uint64_t *out, uint64_t *request_id);
/* Up to `max` completed requests (waits up to timeout_ms for the first). */
int fheacc_server_poll(fheacc_server *srv, fheacc_request_done *done, size_t max, size_t *n_done, uint32_t timeout_ms);
int fheacc_server_stats(fheacc_server *srv, fheacc_server_stats_t *stats);
int fheacc_server_destroy(fheacc_server *srv);

/* ------------------------------------------------- automorphism and expand
 * DEVICE buffers of canonical NTT-domain RLWEs ([count][2N] words),
 * asynchronous on `stream`. f is the substitution factor: X -> X^(N/2^f + 1),
 * 0 <= f < log2 N. */
/* RLWE_substitute (RLWE.cpp:444-462). */
int fheacc_rlwe_substitute_async(fheacc_ctx *ctx, const uint64_t *d_in, size_t count, int f, uint64_t *d_out,
                                 void *stream);
/* RLWE_keyswitch (RLWE.cpp:464-510) of every input with one key given in the
 * reference layout [digitKS_R][2][N] (device words). */
int fheacc_rlwe_keyswitch_async(fheacc_ctx *ctx, const uint64_t *d_in, size_t count, const uint64_t *d_ksk,
                                uint64_t *d_out, void *stream);
/* RLWE_keyswitch(RLWE_substitute(c, f), subs_key[f]) with the uploaded
 * substitute key: the FPGA's RLWESUBS instruction (myfpga.cpp:1708-1745). */
int fheacc_subs_keyswitch_async(fheacc_ctx *ctx, const uint64_t *d_in, size_t count, int f, uint64_t *d_out,
                                void *stream);
/* application::expand_RLWE (app.cpp:26-76): d_out = [N] RLWEs. Replaces
 * fpga_expand_RLWE (myfpga.cpp:1662-1790). Needs the substitute key. */
int fheacc_expand_rlwe(fheacc_ctx *ctx, const uint64_t *d_in, uint64_t *d_out, void *stream);

/* Wait until the most recent asynchronous call of the context (and every
 * blocking call) has finished, at most timeout_ms (0 = no limit). Returns
 * FHEACC_EIO if a kernel of the context flagged its results invalid (see
 * fheacc_device_status). */
int fheacc_sync(fheacc_ctx *ctx, uint32_t timeout_ms);

/* Device status of the context, read and cleared (call after the work has
 * finished). Bit FHEACC_STATUS_WAIT_LIMIT: a blind-rotation worker gave up a
 * bounded wait on another worker of its CTA (every such wait ends within a few
 * steps by construction; the bound keeps a fault from hanging the GPU), and
 * the launch's results are invalid; the call then returns FHEACC_EIO.
 * fheacc_bootstrap and fheacc_sync check it themselves. */
#define FHEACC_STATUS_WAIT_LIMIT 1u
int fheacc_device_status(fheacc_ctx *ctx, uint32_t *bits);

/* Kernels the context has launched since its creation, counting a kernel
 * captured into a CUDA graph once (at capture, not per replay); *count = the
 * total. Reading it around a call gives the number of kernels the call
 * launched. */
int fheacc_kernel_launches(const fheacc_ctx *ctx, uint64_t *count);

#ifdef __cplusplus
}
#endif
#endif
