// ctx.hpp -- the device context behind fheacc_ctx and the launchers shared by
// the kernel translation units. Internal to libfheacc.so.
#pragma once
#include <cuda_runtime.h>
#include <atomic>
#include <cstdint>
#include <string>
#include "fheacc.h"
#include "ntt32.cuh"
#include "ntt64.cuh"
#include "window.cuh"

namespace fheacc {

// Device copy of the parameters the kernels read.
struct DevParams {
    int n, N, logN;
    uint32_t q, embed;          // embed = 2N / q
    uint64_t Q;
    uint32_t BG_bits, digitG, Br, digitR, Bks, digitKS, Bks_R_bits, digitKS_R;
    uint64_t gate_constant[8];  // entries 6, 7 are 0 (guard for bad gate codes)
    uint64_t mu64;              // floor(2^64 / Q), Barrett constant
    uint32_t ks_row;            // padded words per LWE key-switch row (>= n+1, multiple of 32)
    // 32-bit path: bootstrap-key words are stored times key_factor = 2^32 N^-1
    // mod Q, so a Montgomery reduction (qinv_neg = -Q^-1 mod 2^32) of the
    // multiply-accumulate sums both reduces them and carries the iNTT's N^-1.
    uint32_t key_factor, qinv_neg;
    // Q < BG^digitG: the gadget digits of a canonical coefficient recompose it
    // exactly, so the last digit's NTT follows from the NTT-domain accumulator
    // (sum_h BG^h NTT(d_h) = acc). The 32-bit key rows are then uploaded as
    // K'_h = K_h - BG^(h-digitG+1) K_last and K'_last = BG^-(digitG-1) K_last,
    // and the blind rotation multiplies the accumulator by K'_last instead of
    // transforming the last digit.
    uint32_t last_digit_from_acc;
};

// Launch-shape choices of the blind-rotation kernel (set by fheacc_set_option
// or picked by fheacc_autotune).
struct Tuning {
    int br_regs_for_3 = -1;   // register budget for 3 CTAs/SM (1 or -1, the default) or 2 (0)
    int br_ctas_per_sm = 0;   // cap on resident CTAs per SM (0: occupancy limit)
    int br_group = 0;         // cap on ciphertexts per CTA and chunk (0: kernel maximum)
    int br_window = -1;       // 64-bit path: steps per bucket of the step window (0: off; -1: default)
    int br_pipes = 0;         // 32-bit path: pipelines per CTA, 1..3 (0: by gates per SM)
    int br_pool = -1;         // 64-bit path: remainder gates shared by all CTAs (0: off; -1: on)
    int debug_wait_limit = -1;   // tests: polls / idle periods before a bounded wait gives up (-1: built-in)
    int ks_tiled = -1;        // 32-bit LWE key switch: tiled form 1 always (scratch allowing), 0 never, -1 by size
    int br_solo = -1;         // 32-bit path: latency form up to this many gates per SM (0: off; -1: default)
};

constexpr size_t kPipeSmemBudget = 220 * 1024;   // dynamic shared memory of one blind-rotation CTA

// Threads of a 32-bit LWE key-switch CTA, four words of a key row each: rows
// of up to n + 1 <= 1024 words.
constexpr int kKsMaxThreads = 256;

constexpr size_t kClaimWords = 64;   // u32 words of claim counters after the blind-rotation accumulators
// 64-bit blind rotation: most remainder gates of a batch that the CTAs share
// item by item (their per-gate state follows the claim words)
constexpr size_t kPool64 = 256;
// Device status bits (Context::d_status): a kernel that gave up a bounded wait
// on another worker of its CTA sets kStatusWaitLimit; its results are not valid.
constexpr unsigned kStatusWaitLimit = FHEACC_STATUS_WAIT_LIMIT;

// Step-window default of the 64-bit path (steps per bucket; a step's key tile,
// values and Shoup companions, is 18 MB).
constexpr int kWindowWide = 1;
constexpr int kWindowCapacity = 4096;   // buckets of the context's counter buffer

#ifdef __CUDACC__
// Issue rule of a blind-rotation step s of one ciphertext (res: its residues,
// one per step): the reference CPU order applies the steps of non-zero
// residue (RLWE.cpp:759); mode 1 (FHEACC_FLAG_FPGA_X1) also the first step
// (myfpga.cpp:1037-1046); mode 2 (FHEACC_FLAG_FPGA_COMPAT) every step
// (myfpga.cpp:1200-1210).
__device__ __forceinline__ bool step_issued(const uint8_t *res, int s, int mode)
{
    return mode == 2 || res[s] != 0 || (mode == 1 && s == 0);
}
// The issue mode of a call's flags.
__host__ __device__ __forceinline__ int issue_mode(uint32_t flags)
{
    return (flags & FHEACC_FLAG_FPGA_COMPAT) ? 2 : (flags & FHEACC_FLAG_FPGA_X1) ? 1 : 0;
}
#endif

// Makes `dev` current for a scope and restores the caller's device.
struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev)
    {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard()
    {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

struct Scratch {
    void *ptr = nullptr;
    size_t bytes = 0;
};

struct Context {
    fheacc_params p{};
    DevParams dp{};
    int device = 0;
    bool wide = false;            // 64-bit path: N = 2048, Q < 2^58 (else N = 1024, Q < 2^27)
    cudaStream_t stream = nullptr;  // used by the blocking host-buffer entry points
    cudaEvent_t done = nullptr;     // recorded after every asynchronous call
    cudaEvent_t prof[3] = {nullptr, nullptr, nullptr};   // FHEACC_FLAG_PROFILE marks
    std::string err;
    Tuning tune;

    // twiddles: (w, w') pairs indexed like the reference tables
    uint2 *d_fwd_tw = nullptr, *d_inv_tw = nullptr;
    dev::Ntt32Consts nc{};

    // 64-bit path: twiddles as (w, floor(w 2^64 / Q)) pairs in reference order
    ulonglong2 *d_tw64 = nullptr, *d_itw64 = nullptr;
    dev::Ntt64Consts nc64{};
    ulonglong2 *d_btkey64 = nullptr;   // Shoup pairs, [(i*digitR + j)*Br + r][digitG][2][2][N]
    ulonglong2 *d_cf64 = nullptr;      // factors of the last-digit identity, digitG Shoup pairs
    ulonglong2 *d_subs64 = nullptr;    // Shoup pairs, [logN][digitKS_R][2][N]
    uint64_t *d_rot = nullptr;         // [logN][N]: NTT(-X^(N - 2^j)), rotate_vector_gen(false)
    uint64_t *d_rot_fwd = nullptr;     // [logN][N]: NTT(X^(2^j)), rotate_vector_gen(true)
    uint64_t *d_kskey64 = nullptr;     // [(d*digitKS + j)*N + i][ks_row]

    // keys, device layouts
    uint32_t *d_btkey = nullptr;   // [(i*digitR + j)*Br + r][digitG][2][2][N], polys B-tiled
    size_t btkey_bytes = 0;
    uint32_t *d_kskey = nullptr;   // [(d*digitKS + j)*N + i][ks_row]
    size_t kskey_bytes = 0;
    uint32_t *d_subs = nullptr;    // [logN][digitKS_R][2][N]
    size_t subs_bytes = 0;

    // scratch owned by the context, grown on demand
    Scratch accs;                  // blind-rotation accumulators, [count][2][N] u32
    Scratch extract;               // extracted RLWEs between blind rotation and key switch
    Scratch io;                    // device staging for the host-buffer entry points
    Scratch psi;                   // CMUX / blind-rotation / homo_expand intermediates (psi.cu)
    Scratch expand;                // shares of the split expand_RLWE levels (expand.cu)
    unsigned *d_window = nullptr;  // step-window counters, kWindowCapacity + 1 (window.cuh)
    unsigned *d_status = nullptr;  // device status word (kStatus*), after the window counters
    std::atomic<uint64_t> launches{0};   // kernels launched (or captured into a graph) so far;
                                         // atomic: a server's worker thread launches while others read

    size_t device_bytes() const
    {
        return btkey_bytes + kskey_bytes + subs_bytes + accs.bytes + extract.bytes + io.bytes + psi.bytes +
               expand.bytes + 2 * (size_t)p.N * sizeof(uint2);
    }
    int fail(int code, const std::string &msg)
    {
        err = msg;
        return code;
    }
    int cuda_fail(cudaError_t e, const char *where)
    {
        err = std::string(where) + ": " + cudaGetErrorString(e);
        return FHEACC_EIO;
    }
};

// Grows `s` to at least `bytes` (device memory).
int ensure_scratch(Context &c, Scratch &s, size_t bytes);

// Step window of a blind-rotation launch over `steps` refresh steps: zeroes
// the context's counters on `st` and fills `w` (w.count null: no window).
int prepare_window(Context &c, int steps, cudaStream_t st, dev::StepWindow &w);

// launchers (bootstrap32.cu)
int launch_ntt32(Context &c, uint64_t *d_polys, size_t count, bool inverse, cudaStream_t st);
// RLWE_mult_RGSW of count accumulators (canonical NTT RLWEs, u64); RGSW i at
// d_rgsw + i * rgsw_stride words (reference layout; stride 0: one shared RGSW).
int launch_rlwe_mult_rgsw32(Context &c, const uint64_t *d_acc, const uint64_t *d_rgsw, uint64_t *d_out,
                            size_t count, size_t rgsw_stride, cudaStream_t st);
// Blind rotation; writes either NTT accumulators (d_acc_out, [count][2N] u64)
// or the extracted time-domain RLWE for the key switch (d_extract, u32
// [count][N + 32]: a[N] after NTT_a_transpose, then b[0]).
int launch_blind_rotate32(Context &c, const uint64_t *d_c1, const uint64_t *d_c2, const int32_t *d_gates,
                          size_t count, uint32_t flags, uint64_t *d_acc_out, uint32_t *d_extract,
                          int max_ctas, cudaStream_t st);
// The same blind rotation writing extracted RLWEs, with caller-supplied
// accumulator scratch (bootstrap_accs_bytes); performs no allocation.
int launch_blind_rotate32_with(Context &c, const uint64_t *d_c1, const uint64_t *d_c2, const int32_t *d_gates,
                               size_t count, uint32_t flags, uint32_t *accs, uint32_t *d_extract, cudaStream_t st);
// Blind rotation whose gate g reads c1 + idx1[g] * (n+1) and c2 + idx2[g] *
// (n+1) (index arrays optional), caller-supplied accumulator scratch.
int launch_blind_rotate32_indexed(Context &c, const uint64_t *d_c1, const uint64_t *d_c2, const uint32_t *d_idx1,
                                  const uint32_t *d_idx2, const int32_t *d_gates, size_t count, uint32_t flags,
                                  uint32_t *accs, uint32_t *d_extract, cudaStream_t st);
// Key switch writing ciphertext ci to d_out + out_idx[ci] * (n+1) (optional).
int launch_lwe_keyswitch32_indexed(Context &c, const uint32_t *d_extract, size_t count, bool modswitch,
                                   uint64_t *d_out, const uint32_t *d_out_idx, cudaStream_t st);
// LWE key switch (+ optional modulus switch) from extracted RLWEs
// (lwe_ks.cu). d_scratch (optional, scratch_bytes of free device memory, 16-byte
// aligned; the blind rotation's accumulators once it is done) lets a few
// ciphertexts' rows be split over many CTAs (count * ks_row u64 words of
// partial sums) and large batches take the tiled form (their digits,
// N * digitKS bytes per gate).
int launch_lwe_keyswitch32(Context &c, const uint32_t *d_extract, size_t count, bool modswitch, uint64_t *d_out,
                           cudaStream_t st, void *d_scratch = nullptr, size_t scratch_bytes = 0,
                           const uint32_t *d_out_idx = nullptr);
// Batches from this many gates take the tiled key switch.
constexpr size_t kKsTiledMinGates = 1024;
int launch_extract_from_ntt32(Context &c, const uint64_t *d_rlwe, size_t count, uint32_t *d_extract,
                              cudaStream_t st);
int launch_modswitch(Context &c, const uint64_t *d_in, size_t count, uint64_t *d_out, cudaStream_t st);
// 64-bit path (bootstrap64.cu)
int launch_shoup_pairs64(Context &c, const uint64_t *d_in, ulonglong2 *d_out, size_t n, cudaStream_t st);
// The last-digit identity applied in place to count RGSWs (d_cf: digitG Shoup pairs).
int launch_derive_keys64(Context &c, uint64_t *d_keys, size_t count, const ulonglong2 *d_cf, cudaStream_t st);
int launch_ntt64(Context &c, uint64_t *d_polys, size_t count, bool inverse, cudaStream_t st);
int launch_rlwe_mult_rgsw64(Context &c, const uint64_t *d_acc, const uint64_t *d_rgsw, uint64_t *d_out,
                            size_t count, size_t rgsw_stride, cudaStream_t st);
// expand_RLWE (app.cpp:26-76) of `count` NTT RLWEs (d_in: [count][2N]), each
// into N (d_out: [count][N][2N]), all expansions level by level in one launch
// per level.
int expand_device(Context &c, const uint64_t *d_in, uint64_t *d_out, cudaStream_t st, size_t count = 1);
int launch_blind_rotate64(Context &c, const uint64_t *d_c1, const uint64_t *d_c2, const int32_t *d_gates,
                          size_t count, uint32_t flags, uint64_t *d_acc_out, uint64_t *d_extract, int max_ctas,
                          cudaStream_t st);
// The same with caller-supplied accumulator scratch (count * 4096 u64 words).
int launch_blind_rotate64_with(Context &c, const uint64_t *d_c1, const uint64_t *d_c2, const int32_t *d_gates,
                               size_t count, uint32_t flags, uint64_t *accs, uint64_t *d_acc_out,
                               uint64_t *d_extract, int max_ctas, cudaStream_t st);
int launch_extract64(Context &c, const uint64_t *d_rlwe, size_t count, uint64_t *d_extract, cudaStream_t st);
// Tiled 64-bit LWE key switch (lwe_ks.cu): whether it applies to `count` gates
// with `scratch_bytes` of scratch for the digits, and the launch.
bool ks64_tiled_applies(const Context &c, size_t count, int sms, size_t scratch_bytes);
int launch_ks64_tiled(Context &c, const uint64_t *d_extract, size_t count, bool modswitch, uint64_t *d_out,
                      const uint32_t *d_out_idx, void *scratch, int sms, cudaStream_t st);
// d_scratch (optional, scratch_bytes of free device memory): from two gates
// per SM holds the tiled form's digits; below, lets a few ciphertexts' rows be
// split over many CTAs (count * ks_row u64 partial sums).
int launch_lwe_keyswitch64(Context &c, const uint64_t *d_extract, size_t count, bool modswitch, uint64_t *d_out,
                           cudaStream_t st, const uint32_t *d_out_idx = nullptr, void *d_scratch = nullptr,
                           size_t scratch_bytes = 0);
// The 64-bit blind rotation reading gate g's inputs at c1 + idx1[g] * (n+1)
// and c2 + idx2[g] * (n+1) (index arrays optional), caller-supplied
// accumulator scratch (bootstrap_accs_bytes); window = false takes no step
// window (for launches that may overlap another launch of the context).
int launch_blind_rotate64_indexed(Context &c, const uint64_t *d_c1, const uint64_t *d_c2, const uint32_t *d_idx1,
                                  const uint32_t *d_idx2, const int32_t *d_gates, size_t count, uint32_t flags,
                                  uint64_t *accs, uint64_t *d_acc_out, uint64_t *d_extract, int max_ctas,
                                  bool window, cudaStream_t st);
// automorphism / key switch / expand (expand.cu); mode: 0 SUBS, 1 KS,
// 2 SUBS_KS, 3 EXPAND (one level f, in place on d_out, for `batches` r
// arrays bstride words apart)
int launch_expand(Context &c, int mode, const uint64_t *d_in, uint64_t *d_out, size_t count, int f,
                  const void *ksk, const uint64_t *d_rot, cudaStream_t st, size_t batches = 1, size_t bstride = 0);
int launch_to_u32(Context &c, const uint64_t *d_in, uint32_t *d_out, size_t n, cudaStream_t st);
// IMAD throughput probe (probe.cu)
int measure_imad_rate(Context &c, double *imad_per_s);
int measure_components(Context &c, double ns[4]);
int measure_l2_read_rate(Context &c, double *bytes_per_s);

constexpr size_t kExtractStride = 1024 + 32;   // u32 words per extracted RLWE (N = 1024)
constexpr size_t kExtract64 = 2048 + 8;        // u64 words per extracted RLWE (N = 2048)

// Device scratch of one batched bootstrap of `count` gates: blind-rotation
// accumulators and extracted RLWEs (bytes of each).
inline size_t bootstrap_accs_bytes(const Context &c, size_t count)
{
    return c.wide ? count * 4096 * sizeof(uint64_t) + kClaimWords * sizeof(uint32_t) +
                        kPool64 * (2 * sizeof(int) + (size_t)c.p.n * c.p.digitR)
                  : (count * 2048 + kClaimWords) * sizeof(uint32_t);
}
inline size_t bootstrap_extract_bytes(const Context &c, size_t count)
{
    return c.wide ? count * kExtract64 * sizeof(uint64_t) : count * kExtractStride * sizeof(uint32_t);
}
// Batched gate bootstrap (blind rotation, key switch, modulus switch) on `st`
// with caller-supplied scratch of the sizes above; no allocation, no host
// synchronisation, so it can be captured into a CUDA graph (api.cu).
int bootstrap_device_with(Context &c, const uint64_t *d_c1, const uint64_t *d_c2, const int32_t *d_gates,
                          size_t count, uint64_t *d_out, uint32_t flags, void *accs, void *extract,
                          cudaStream_t st);
// The same with the context's own scratch (grown on demand).
int bootstrap_device(Context &c, const uint64_t *d_c1, const uint64_t *d_c2, const int32_t *d_gates,
                     size_t count, uint64_t *d_out, uint32_t flags, cudaStream_t st, int max_ctas);

// Word index of element e = 32 l + r of a 1024-word poly in the "B-tiled"
// device layout used for bootstrap keys and blind-rotation accumulators.
inline size_t btile_index(size_t e)
{
    const size_t l = e >> 5, r = e & 31;
    return (((r >> 2) << 5) + l) * 4 + (r & 3);
}

}  // namespace fheacc
