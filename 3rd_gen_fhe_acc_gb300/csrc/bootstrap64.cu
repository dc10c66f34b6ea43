// bootstrap64.cu -- the 64-bit-word path: N = 2048 and Q < 2^58 (the
// n=630, Q < 2^54, BG = 2^9 x 6 parameter set), blind rotation, NTT and
// RLWE x RGSW sub-steps, extraction, LWE key switch and modulus switch.
//
// Reference behaviour as in the 32-bit path: eval_bootstrap
// (FHE_ACC_runtime/src/RLWE.cpp:726-786), RLWE_mult_RGSW (RLWE.cpp:642-704),
// digit_decompose (RLWE.cpp:623-640), acc_initialization (RLWE.cpp:706-724),
// LWE_keyswitch / LWE_modswitch (LWE.cpp:233-269).
//
// One RLWE x RGSW step runs on a CTA of 256 threads in two 128-thread groups,
// group p owning poly p of the accumulator: inverse NTT in shared memory, then
// for each digit h both groups transform digit h of their poly and all 256
// threads multiply-accumulate it with the key rows. Keys are stored with their
// Shoup companions (K, floor(K 2^64 / Q)), so every MAC product is one 64-bit
// Shoup multiply; the 2 * digitG products of an output stay below 24Q and are
// reduced once. As in the 32-bit kernel, steps are the outer loop over a
// group of ciphertexts per CTA, so the CTAs stream each step's 23 RGSW keys
// (18 MB with companions) through L2 together; accumulators live in global
// memory (32 KB per gate).
#include "ctx.hpp"
#include "l2hint.cuh"
#include "ntt64.cuh"
#include <algorithm>

namespace fheacc {
namespace dev {

constexpr int kMaxGroup64 = 8;   // ciphertexts per worker and claim
constexpr int kT64 = 256;   // threads per CTA

// One worker's polys in shared memory, layout pi<P> (ntt64.cuh): padded in the
// blind rotation, plain in the RLWE x RGSW kernel (whose L1 the padding costs).
template <bool P>
struct Step64SmemT {
    uint64_t acc[2][poly_words64<P>()];   // accumulator; time domain inside a step
    uint64_t buf[2][poly_words64<P>()];   // digit NTTs
};

constexpr int kMaxTableBG64 = 512;   // largest gadget base with digit tables (40 BG bytes of shared memory)

__device__ __forceinline__ uint64_t mulmod64(uint64_t a, uint64_t b, uint64_t Q)
{
    return (uint64_t)((unsigned __int128)a * b % Q);
}

// Builds the digit tables (DigitTables64) for y < BG in `mem` (40 BG bytes,
// 16-byte aligned) from the twiddles tw[1..3]; all threads of the CTA take part.
__device__ __forceinline__ DigitTables64 build_digit_tables64(unsigned char *mem, int BG,
                                                             const ulonglong2 *__restrict__ tw, uint64_t Q)
{
    ulonglong2 *t23 = reinterpret_cast<ulonglong2 *>(mem), *t123 = t23 + BG;
    uint64_t *t1 = reinterpret_cast<uint64_t *>(t123 + BG);
    const uint64_t w1 = tw[1].x, w2 = tw[2].x, w3 = tw[3].x;
    const uint64_t w21 = mulmod64(w2, w1, Q), w31 = mulmod64(w3, w1, Q);
    for (int y = threadIdx.x; y < BG; y += blockDim.x) {
        t1[y] = mulmod64((uint64_t)y, w1, Q);
        t23[y] = make_ulonglong2(mulmod64((uint64_t)y, w2, Q), mulmod64((uint64_t)y, w3, Q));
        t123[y] = make_ulonglong2(mulmod64((uint64_t)y, w21, Q), mulmod64((uint64_t)y, w31, Q));
    }
    return DigitTables64{t1, t23, t123};
}

// One RLWE x RGSW step on s.acc (NTT domain, values < 2Q) with the key
// `key` (Shoup pairs, [digitG][2][2][2048]), run by the 256 threads tid of a
// worker that synchronises on named barrier `bar` (its two 128-thread groups
// on bar + 1 and bar + 2).
// With acc_nd (the step's NTT-domain accumulator in global memory, read before
// it is overwritten) the last digit's NTT is replaced by the accumulator: the
// keys were uploaded with K'_h = K_h - BG^(h-DG+1) K_last, K'_last =
// BG^-(DG-1) K_last (Q < BG^DG, so sum_h BG^h NTT(digit_h) = acc).
// With dt the digit transforms start from the digit tables (BG <= kMaxTableBG64).
// KEEP: acc_nd is read with the L2 evict-last policy (l2hint.cuh).
template <bool P, bool KEEP = false>
__device__ __forceinline__ void step64(Step64SmemT<P> &s, const ulonglong2 *__restrict__ key, int DG, uint32_t bg_bits,
                                       const ulonglong2 *__restrict__ tw, const ulonglong2 *__restrict__ itw,
                                       const Ntt64Consts &c, const uint64_t *acc_nd, int tid, int bar,
                                       const DigitTables64 *dt = nullptr)
{
    const int grp = tid >> 7, gtid = tid & 127;
    ntt64_inv_2048<128, P>(s.acc[grp], itw, c, gtid, bar + 1 + grp);
    group_sync(bar, kT64);
    uint64_t sa[8], sb[8];
#pragma unroll
    for (int i = 0; i < 8; i++) sa[i] = sb[i] = 0;
    const uint64_t mask = (1ULL << bg_bits) - 1;
    const int DH = acc_nd ? DG - 1 : DG;   // digits transformed
    for (int h = 0; h < DH; h++) {
        const uint32_t sh = bg_bits * h;
        for (int e = gtid; e < 2048; e += 128) s.buf[grp][pi<P>(e)] = (s.acc[grp][pi<P>(e)] >> sh) & mask;
        group_sync(bar + 1 + grp, 128);
        if (dt) ntt64_fwd_2048_digit<128, P>(s.buf[grp], tw, c, gtid, bar + 1 + grp, *dt);
        else ntt64_fwd_2048<128, P>(s.buf[grp], tw, c, gtid, bar + 1 + grp);
        group_sync(bar, kT64);
        const ulonglong2 *k0 = key + (size_t)(h * 2 + 0) * 2 * 2048;   // row c_text[h][0]: times digit of a
        const ulonglong2 *k1 = key + (size_t)(h * 2 + 1) * 2 * 2048;   // row c_text[h][1]: times digit of b
#pragma unroll
        for (int i = 0; i < 8; i++) {
            const int k = tid + 256 * i;
            const uint64_t da = s.buf[0][pi<P>(k)], db = s.buf[1][pi<P>(k)];
            const ulonglong2 a0 = __ldg(k0 + k), b0 = __ldg(k0 + 2048 + k);
            const ulonglong2 a1 = __ldg(k1 + k), b1 = __ldg(k1 + 2048 + k);
            sa[i] += shoup64(da, a0.x, a0.y, c.Q) + shoup64(db, a1.x, a1.y, c.Q);
            sb[i] += shoup64(da, b0.x, b0.y, c.Q) + shoup64(db, b1.x, b1.y, c.Q);
        }
        group_sync(bar, kT64);
    }
    if (acc_nd) {
        const ulonglong2 *k0 = key + (size_t)((DG - 1) * 2 + 0) * 2 * 2048;
        const ulonglong2 *k1 = key + (size_t)((DG - 1) * 2 + 1) * 2 * 2048;
#pragma unroll
        for (int i = 0; i < 8; i++) {
            const int k = tid + 256 * i;
            uint64_t da, db;
            if (KEEP) {
                const uint64_t pol = l2_keep_policy();
                da = ld_keep64(acc_nd + k, pol);
                db = ld_keep64(acc_nd + 2048 + k, pol);
            } else {
                da = __ldcg(acc_nd + k);
                db = __ldcg(acc_nd + 2048 + k);
            }
            const ulonglong2 a0 = __ldg(k0 + k), b0 = __ldg(k0 + 2048 + k);
            const ulonglong2 a1 = __ldg(k1 + k), b1 = __ldg(k1 + 2048 + k);
            sa[i] += shoup64(da, a0.x, a0.y, c.Q) + shoup64(db, a1.x, a1.y, c.Q);
            sb[i] += shoup64(da, b0.x, b0.y, c.Q) + shoup64(db, b1.x, b1.y, c.Q);
        }
    }
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int k = tid + 256 * i;
        s.acc[0][pi<P>(k)] = barrett64_2q(sa[i], c.mu64, c.Q);
        s.acc[1][pi<P>(k)] = barrett64_2q(sb[i], c.mu64, c.Q);
    }
    group_sync(bar, kT64);
}

// Forward / inverse NTT of count polys (u64, canonical in and out), one
// 128-thread group per poly.
template <bool INV>
__global__ void __launch_bounds__(kT64) ntt64_kernel(uint64_t *polys, size_t count, const ulonglong2 *__restrict__ tw,
                                                    const __grid_constant__ Ntt64Consts c)
{
    __shared__ uint64_t buf[2][2048];
    const int grp = threadIdx.x >> 7, gtid = threadIdx.x & 127;
    for (size_t base = (size_t)blockIdx.x * 2; base < count; base += (size_t)gridDim.x * 2) {
        const size_t pi = base + grp;
        const bool live = pi < count;
        uint64_t *poly = polys + pi * 2048;
        for (int e = gtid; e < 2048; e += 128) buf[grp][e] = live ? poly[e] : 0;
        group_sync(1 + grp, 128);
        if (INV) ntt64_inv_2048<128, false>(buf[grp], tw, c, gtid, 1 + grp);
        else ntt64_fwd_2048<128, false>(buf[grp], tw, c, gtid, 1 + grp);
        if (live) {
            for (int e = gtid; e < 2048; e += 128) {
                uint64_t v = buf[grp][e];
                if (!INV) {
                    v = barrett64_2q(v, c.mu64, c.Q);
                    v = v >= c.Q ? v - c.Q : v;
                }
                poly[e] = v;
            }
        }
        __syncthreads();
    }
}

// The last-digit identity on `count` RGSWs [DG][4][N] (u64, reduced in
// place): row h < DG-1 becomes K_h - cf[h] K_last, row DG-1 becomes
// cf[DG-1] K_last, mod Q; (cf, cfs) Shoup pairs of the factors.
__global__ void derive_keys64_kernel(uint64_t *__restrict__ keys, size_t count, int DG, int N,
                                     const ulonglong2 *__restrict__ cf, uint64_t Q)
{
    const size_t plane = 4 * (size_t)N;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < count * plane;
         i += (size_t)gridDim.x * blockDim.x) {
        const size_t g = i / plane, x = i - g * plane;
        uint64_t *rg = keys + g * (size_t)DG * plane;
        const uint64_t last = rg[(size_t)(DG - 1) * plane + x] % Q;
        for (int h = 0; h + 1 < DG; h++) {
            const uint64_t k = rg[(size_t)h * plane + x] % Q;
            uint64_t m = shoup64(last, cf[h].x, cf[h].y, Q);
            m = m >= Q ? m - Q : m;
            rg[(size_t)h * plane + x] = k >= m ? k - m : k + Q - m;
        }
        uint64_t m = shoup64(last, cf[DG - 1].x, cf[DG - 1].y, Q);
        rg[(size_t)(DG - 1) * plane + x] = m >= Q ? m - Q : m;
    }
}

// (K, floor(K 2^64 / Q)) pairs of key words (reduced mod Q first).
__global__ void shoup_pairs64_kernel(const uint64_t *__restrict__ in, ulonglong2 *__restrict__ out, size_t n,
                                     uint64_t Q)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const uint64_t w = in[i] % Q;
        out[i] = make_ulonglong2(w, (uint64_t)(((unsigned __int128)w << 64) / Q));
    }
}

// RLWE_mult_RGSW of count (acc, RGSW-pairs) in reference order; acc canonical.
// derive: the RGSWs carry the last-digit identity (derive_keys64_kernel) and the
// last digit's NTT is the input accumulator itself.
__global__ void __launch_bounds__(kT64) rlwe_mult_rgsw64_kernel(const uint64_t *__restrict__ acc_in,
                                                               const ulonglong2 *__restrict__ rgsw, uint64_t *acc_out,
                                                               size_t count, size_t rgsw_stride, int DG, uint32_t bg_bits,
                                                               const ulonglong2 *__restrict__ tw,
                                                               const ulonglong2 *__restrict__ itw,
                                                               const __grid_constant__ Ntt64Consts c, int derive)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Step64SmemT<false> &s = *reinterpret_cast<Step64SmemT<false> *>(smem_raw);
    for (size_t ci = blockIdx.x; ci < count; ci += gridDim.x) {
        for (int e = threadIdx.x; e < 4096; e += kT64) s.acc[e >> 11][e & 2047] = acc_in[ci * 4096 + e];
        __syncthreads();
        step64(s, rgsw + ci * rgsw_stride, DG, bg_bits, tw, itw, c, derive ? acc_in + ci * 4096 : nullptr,
               threadIdx.x, 1);
        for (int e = threadIdx.x; e < 4096; e += kT64) {
            const uint64_t v = s.acc[e >> 11][e & 2047];
            acc_out[ci * 4096 + e] = v >= c.Q ? v - c.Q : v;
        }
        __syncthreads();
    }
}

// RLWE x RGSW of a few products, split over the gadget digits for latency: CTA
// (product ci, digit h) takes the inverse NTT of the product's accumulator,
// digit h of both polys and their forward NTTs, and writes the digit's share of
// the multiply-accumulate to partial[ci][h] (two Shoup products per word, < 4Q);
// rlwe_split_sum64_kernel adds the digitG shares. A lone product's inverse and
// digit NTTs then take two rounds instead of 1 + digitG.
__global__ void __launch_bounds__(kT64) rlwe_mult_rgsw64_split_kernel(const uint64_t *__restrict__ acc_in,
                                                                     const ulonglong2 *__restrict__ rgsw,
                                                                     uint64_t *__restrict__ partial, size_t rgsw_stride,
                                                                     int DG, uint32_t bg_bits,
                                                                     const ulonglong2 *__restrict__ tw,
                                                                     const ulonglong2 *__restrict__ itw,
                                                                     const __grid_constant__ Ntt64Consts c)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Step64SmemT<false> &s = *reinterpret_cast<Step64SmemT<false> *>(smem_raw);
    const size_t ci = blockIdx.x / (unsigned)DG;
    const int h = (int)(blockIdx.x - ci * (unsigned)DG);
    const int tid = threadIdx.x, grp = tid >> 7, gtid = tid & 127;
    for (int e = tid; e < 4096; e += kT64) s.acc[e >> 11][e & 2047] = acc_in[ci * 4096 + e];
    __syncthreads();
    ntt64_inv_2048<128, false>(s.acc[grp], itw, c, gtid, 2 + grp);   // ends with the group's barrier
    const uint64_t mask = (1ULL << bg_bits) - 1;
    const uint32_t sh = bg_bits * (uint32_t)h;
    for (int e = gtid; e < 2048; e += 128) s.buf[grp][e] = (s.acc[grp][e] >> sh) & mask;
    group_sync(2 + grp, 128);
    ntt64_fwd_2048<128, false>(s.buf[grp], tw, c, gtid, 2 + grp);
    __syncthreads();
    const ulonglong2 *key = rgsw + ci * rgsw_stride;
    const ulonglong2 *k0 = key + (size_t)(h * 2 + 0) * 2 * 2048;   // row c_text[h][0]: times digit of a
    const ulonglong2 *k1 = key + (size_t)(h * 2 + 1) * 2 * 2048;   // row c_text[h][1]: times digit of b
    uint64_t *out = partial + (ci * (unsigned)DG + (unsigned)h) * 4096;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int k = tid + 256 * i;
        const uint64_t da = s.buf[0][k], db = s.buf[1][k];
        const ulonglong2 a0 = __ldg(k0 + k), b0 = __ldg(k0 + 2048 + k);
        const ulonglong2 a1 = __ldg(k1 + k), b1 = __ldg(k1 + 2048 + k);
        out[k] = shoup64(da, a0.x, a0.y, c.Q) + shoup64(db, a1.x, a1.y, c.Q);
        out[2048 + k] = shoup64(da, b0.x, b0.y, c.Q) + shoup64(db, b1.x, b1.y, c.Q);
    }
}

// acc_out[ci] = sum over h of partial[ci][h] mod Q (canonical); the sum of
// digitG shares < 4Q stays below 2^64 (checked by the launcher).
__global__ void rlwe_split_sum64_kernel(const uint64_t *__restrict__ partial, uint64_t *__restrict__ acc_out,
                                        size_t count, int DG, const __grid_constant__ Ntt64Consts c)
{
    const size_t words = count * 4096;
    for (size_t w = (size_t)blockIdx.x * blockDim.x + threadIdx.x; w < words; w += (size_t)gridDim.x * blockDim.x) {
        const size_t ci = w / 4096, e = w - ci * 4096;
        const uint64_t *p = partial + ci * (unsigned)DG * 4096 + e;
        uint64_t sum = 0;
        for (int h = 0; h < DG; h++) sum += p[(size_t)h * 4096];
        const uint64_t v = barrett64_2q(sum, c.mu64, c.Q);
        acc_out[w] = v >= c.Q ? v - c.Q : v;
    }
}

struct Br64Args {
    const uint64_t *c1, *c2;
    const uint32_t *idx1, *idx2;   // optional: gate g reads c1 + idx1[g] * (n+1) (else g)
    const int32_t *gates;
    size_t count;
    const ulonglong2 *btkey;   // [(i*digitR + j)*Br + r][digitG][2][2][2048] Shoup pairs
    uint64_t *accs;            // scratch [count][2][2048], NTT domain, values < 2Q
    uint64_t *acc_out;         // optional canonical NTT accumulators [count][4096]
    uint64_t *extract;         // optional [count][kExtract64]
    int group;                 // ciphertexts per claim (<= kMaxGroup64 per worker)
    int derive_last;           // last digit's NTT from the accumulator (DevParams::last_digit_from_acc)
    int n, DG;
    uint32_t q, embed, Br, digitR, bg_bits, flags;
    uint64_t gate_constant[8];
    StepWindow win;            // keeps the CTAs within a few steps of each other (window.cuh)
    unsigned long long *claim_next;   // next unclaimed ciphertext (zeroed before the launch)
    unsigned *status;          // set to kStatusWaitLimit if a worker gave up waiting
    unsigned wait_limit;       // polls before such a wait gives up (kWorkerWaitLimit)
    int digit_tables;          // digit NTTs start from tables (DigitTables64) after the residues
    size_t claim_limit;        // ciphertexts [0, claim_limit) are claimed in groups
    // remainder pool: ciphertexts [pool_first, pool_first + pool_count) that all
    // CTAs share item by item (0: none); their state after the claim words
    int pool_count;
    size_t pool_first;
    unsigned long long *pool_cursor;   // next (step, pool ciphertext) item, step-major (zeroed)
    int *pool_done;            // [pool_count] last finished step (-1: none yet)
    int *pool_last;            // [pool_count] last step with a non-zero residue (-1: none)
    uint8_t *pool_res;         // [pool_count][n * digitR] residues
};

// LWE_evaluate (LWE.cpp:203-222) of ciphertext gid and the residues of its
// refresh steps, the base-Br digits of (q - a_i) mod q (RLWE.cpp:740-760), into
// res[n * digitR]; the thread that takes i = n writes the b value and the gate's
// two test-vector bounds. Threads t0, t0 + nt, ... take part.
__device__ __forceinline__ void br64_residues(const Br64Args &A, size_t gid, uint8_t *res, uint32_t *bval,
                                              uint32_t *b1, uint32_t *b2, int t0, int nt)
{
    const int n = A.n;
    const uint32_t q = A.q, qmask = q - 1;
    const int g = A.gates[gid];
    const bool x2 = (g == 4 || g == 5);
    const uint64_t *c1 = A.c1 + (A.idx1 ? (size_t)A.idx1[gid] : gid) * (size_t)(n + 1);
    const uint64_t *c2 = A.c2 + (A.idx2 ? (size_t)A.idx2[gid] : gid) * (size_t)(n + 1);
    for (int i = t0; i <= n; i += nt) {
        const uint64_t v = x2 ? 2 * (c1[i] - c2[i]) : c1[i] + c2[i];
        if (i < n) {
            uint32_t nega = (q - (uint32_t)(v & qmask)) & qmask;
            for (uint32_t j = 0; j < A.digitR; j++) {
                res[i * (int)A.digitR + (int)j] = (uint8_t)(nega % A.Br);
                nega /= A.Br;
            }
        } else {
            const uint64_t gc = A.gate_constant[(unsigned)g < 6u ? g : 6];
            *bval = (uint32_t)(v & qmask);
            *b1 = (uint32_t)(gc & qmask);
            *b2 = (*b1 + q / 2) & qmask;
        }
    }
}

// acc_initialization (RLWE.cpp:706-724) of ciphertext gid into its accumulator:
// a = 0, b = the test vector, forward NTT. buf: a shared poly (layout pi<P>)
// that the worker's second 128-thread group transforms; bar: the worker's
// barrier (its groups on bar + 1 and bar + 2).
template <bool P>
__device__ __forceinline__ void br64_acc_init(const Br64Args &A, const Ntt64Consts &c, const ulonglong2 *tw,
                                              size_t gid, uint32_t val, uint32_t b1, uint32_t b2, uint64_t *buf,
                                              int tid, int bar)
{
    const uint32_t q = A.q, qmask = q - 1;
    const uint64_t Q8 = c.Q / 8 + 1, negQ8 = c.Q - Q8;
    for (int e = tid; e < 2048; e += kT64) {
        uint64_t v = 0;
        if (e % A.embed == 0 && (uint32_t)e / A.embed < q / 2) {
            const uint32_t tmp = (val - (uint32_t)e / A.embed) & qmask;
            if (b1 < b2) v = (tmp >= b1 && tmp < b2) ? negQ8 : Q8;
            else v = (tmp >= b2 && tmp < b1) ? Q8 : negQ8;
        }
        buf[pi<P>(e)] = v;
    }
    group_sync(bar, kT64);
    if (tid >= 128) ntt64_fwd_2048<128, P>(buf, tw, c, tid - 128, bar + 2);
    group_sync(bar, kT64);
    uint64_t *acc = A.accs + gid * 4096;
    const uint64_t pol = l2_keep_policy();
    for (int e = tid; e < 2048; e += kT64) {
        st_keep64(acc + e, 0, pol);
        const uint64_t v = barrett64_2q(buf[pi<P>(e)], c.mu64, c.Q);
        st_keep64(acc + 2048 + e, v >= c.Q ? v - c.Q : v, pol);
    }
    group_sync(bar, kT64);
}

// Output of ciphertext gid from its accumulator: the extracted RLWE
// (NTT_a_transpose, RLWE.cpp:218-226, then the inverse NTT of both polys) or
// the canonical NTT accumulator. a0, a1: shared polys (layout pi<P>).
template <bool P>
__device__ __noinline__ void br64_output(const Br64Args &A, const Ntt64Consts &c, const ulonglong2 *itw,
                                            size_t gid, uint64_t *a0, uint64_t *a1, int tid, int bar)
{
    const uint64_t *acc = A.accs + gid * 4096;
    if (A.extract) {
        for (int e = tid; e < 2048; e += kT64) {
            a0[pi<P>(e)] = __ldcg(acc + 2047 - e);
            a1[pi<P>(e)] = __ldcg(acc + 2048 + e);
        }
        group_sync(bar, kT64);
        ntt64_inv_2048<128, P>(tid < 128 ? a0 : a1, itw, c, tid & 127, bar + 1 + (tid >> 7));
        group_sync(bar, kT64);
        uint64_t *ext = A.extract + gid * kExtract64;
        for (int e = tid; e < 2048; e += kT64) ext[e] = a0[pi<P>(e)];
        if (tid == 0) ext[2048] = a1[pi<P>(0)];
    } else {
        for (int e = tid; e < 4096; e += kT64) {
            const uint64_t v = __ldcg(acc + e);
            A.acc_out[gid * 4096 + e] = v >= c.Q ? v - c.Q : v;
        }
    }
    group_sync(bar, kT64);
}

// Remainder pool set-up, one 256-thread CTA per pool ciphertext, before the
// blind rotation on the same stream: residues, last non-zero step, the
// initialised accumulator, and the output of a ciphertext without steps.
__global__ void __launch_bounds__(kT64) br64_pool_init_kernel(const __grid_constant__ Br64Args A,
                                                             const ulonglong2 *__restrict__ tw,
                                                             const ulonglong2 *__restrict__ itw,
                                                             const __grid_constant__ Ntt64Consts c)
{
    __shared__ uint64_t buf[2][2048];
    __shared__ uint32_t bv[3];
    __shared__ int last;
    const int p = blockIdx.x, tid = threadIdx.x;
    const int S = A.n * (int)A.digitR;
    const size_t gid = A.pool_first + (size_t)p;
    uint8_t *res = A.pool_res + (size_t)p * S;
    br64_residues(A, gid, res, &bv[0], &bv[1], &bv[2], tid, kT64);
    __syncthreads();
    if (tid == 0) {
        int l = -1;
        const int mode = issue_mode(A.flags);
        for (int x = S - 1; x >= 0; x--)
            if (step_issued(res, x, mode)) {
                l = x;
                break;
            }
        last = l;
        A.pool_last[p] = l;
        A.pool_done[p] = -1;
    }
    br64_acc_init<false>(A, c, tw, gid, bv[0], bv[1], bv[2], buf[1], tid, 1);
    __syncthreads();
    if (last < 0) br64_output<false>(A, c, itw, gid, buf[0], buf[1], tid, 1);
}

// Polls of a worker waiting for another worker's step of the same ciphertext
// (about 60 ns each) before it gives up and flags the launch.
constexpr unsigned kWorkerWaitLimit = 1u << 26;

// Takes the next item of the remainder pool whose step is at most `reach`,
// skipping the items the issue mode skips (step_issued); false when there is none.
// prev: the item's ciphertext's last earlier step with a non-zero residue.
// seen: the CTA's last view of the pool cursor, which only grows, so the
// cursor is read only when the view leaves an item to take.
__device__ __forceinline__ bool pool_take(const Br64Args &A, int S, int mode, unsigned long long reach,
                                          unsigned long long *seen, int &st, int &k, int &prev)
{
    const unsigned long long R = (unsigned long long)A.pool_count, total = R * (unsigned long long)S;
    unsigned long long v = *(volatile unsigned long long *)seen;
    if (v >= total || v / R > reach) return false;
    v = *(volatile unsigned long long *)A.pool_cursor;
    for (;;) {
        if (v >= total || v / R > reach) {
            atomicMax(seen, v);
            return false;
        }
        const unsigned long long old = atomicCAS(A.pool_cursor, v, v + 1);
        if (old != v) {
            v = old;
            continue;
        }
        const int s_ = (int)(v / R), k_ = (int)(v - (unsigned long long)s_ * R);
        const uint8_t *pr = A.pool_res + (size_t)k_ * S;
        if (step_issued(pr, s_, mode)) {
            atomicMax(seen, v + 1);
            st = s_;
            k = k_;
            prev = st - 1;
            while (prev >= 0 && !step_issued(pr, prev, mode)) prev--;
            return true;
        }
        v++;   // an item of zero residue, taken and skipped
    }
}

// W workers of 256 threads per CTA (W = 1: 3 CTAs per SM, 80 registers; the
// extra resident warps hide the latency of the key stream better than the
// spill-free 2-CTA register allocation, 862 vs 1028 ms for 2048 gates). Each
// CTA claims groups of consecutive ciphertexts; its workers share the group's
// (step, ciphertext) items through a cursor that walks them step-major, and a
// worker issues an item once the previous item of its ciphertext (its last
// earlier step with a non-zero residue) has finished, so every ciphertext's
// steps keep the reference's order and the workers finish together. Worker w
// synchronises on named barrier 1 + 3w (its two 128-thread groups on 2 + 3w and
// 3 + 3w). When the batch does not divide evenly among the CTAs, the remainder
// ciphertexts form a pool that all CTAs share item by item (pool_take), their
// steps ordered by done words in global memory. An XOR swizzle of the shared-memory passes removed their bank
// conflicts but cost more in index arithmetic than it saved.
template <int W, int MINB>
__global__ void __launch_bounds__(W * kT64, MINB) br64_kernel(const __grid_constant__ Br64Args A,
                                                          const ulonglong2 *__restrict__ tw,
                                                          const ulonglong2 *__restrict__ itw,
                                                          const __grid_constant__ Ntt64Consts c)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint8_t *res = smem_raw + W * sizeof(Step64SmemT<true>);   // [group][n * digitR]
    __shared__ uint32_t bvals[kMaxGroup64 * W], b1s[kMaxGroup64 * W], b2s[kMaxGroup64 * W];
    __shared__ int done[kMaxGroup64 * W];
    __shared__ int plan[W][3];
    __shared__ int cursor, wcur, won;
    __shared__ unsigned long long pool_seen;
    __shared__ unsigned long long claim_first;
    __shared__ int claim_m;
    const int wk = threadIdx.x / kT64, tid = threadIdx.x - wk * kT64, bar = 1 + 3 * wk;
    Step64SmemT<true> &s = reinterpret_cast<Step64SmemT<true> *>(smem_raw)[wk];
    const int S = A.n * (int)A.digitR;
    const size_t rgsw_pairs = (size_t)A.DG * 4 * 2048;
    const int mode = issue_mode(A.flags);
    const unsigned target = gridDim.x;   // the window is used with one round of claims
    if (threadIdx.x == 0) {
        wcur = 0;
        won = 1;
        pool_seen = 0;
    }
    // digit tables after the residue table of the largest group
    const DigitTables64 dt = build_digit_tables64(res + ((size_t)A.group * S + 15) / 16 * 16,
                                                  A.digit_tables ? 1 << A.bg_bits : 0, tw, c.Q);
    for (;;) {
        if (threadIdx.x == 0) {
            const unsigned long long f = atomicAdd(A.claim_next, (unsigned long long)A.group);
            claim_first = f;
            claim_m = f < A.claim_limit ? (int)min((unsigned long long)A.group, (unsigned long long)A.claim_limit - f) : 0;
        }
        __syncthreads();
        const size_t first = claim_first;
        const int m = claim_m;
        if (m == 0) break;
        // LWE_evaluate and residues
        for (int k = 0; k < m; k++)
            br64_residues(A, first + (size_t)k, res + k * S, bvals + k, b1s + k, b2s + k, threadIdx.x, blockDim.x);
        for (int k = threadIdx.x; k < m; k += blockDim.x) done[k] = -1;
        if (threadIdx.x == 0) cursor = 0;
        __syncthreads();
        // acc_initialization, one ciphertext per worker: a = 0, b = test vector,
        // forward NTT (the worker's group 1 transforms b)
        for (int k = wk; k < m; k += W)
            br64_acc_init<true>(A, c, tw, first + (size_t)k, bvals[k], b1s[k], b2s[k], s.buf[1], tid, bar);
        __syncthreads();
        // blind rotation: the workers take the group's items from the cursor
        for (;;) {
            if (tid == 0) {
                int st = -1, k = -1, prev = -1, pool = 0;
                // an item of the remainder pool of a step this CTA has reached
                // (of any step once the CTA's own items are all issued)
                if (A.pool_count) {
                    const int own = *(volatile int *)&cursor;
                    pool = pool_take(A, S, mode, own < S * m ? (unsigned long long)(own / m) : ~0ull, &pool_seen,
                                     st, k, prev);
                }
                for (; !pool;) {
                    const int idx = atomicAdd(&cursor, 1);
                    if (idx >= S * m) {
                        // own items all issued: the rest of the pool
                        if (A.pool_count) pool = pool_take(A, S, mode, ~0ull, &pool_seen, st, k, prev);
                        break;
                    }
                    const int s_ = idx / m, k_ = idx - s_ * m;
                    if (step_issued(res + k_ * S, s_, mode)) {
                        st = s_;
                        k = k_;
                        prev = st - 1;
                        while (prev >= 0 && !step_issued(res + k * S, prev, mode)) prev--;
                        break;
                    }
                }
                if (!pool && st >= 0 && A.win.count) {
                    // step window: count this CTA into the buckets it has left, then
                    // wait for the slowest CTA
                    const int b = st / A.win.steps;
                    const int old = atomicMax(&wcur, b);
                    for (int x = old; x < b; x++) atomicAdd(A.win.count + x, 1u);
                    int on = won;
                    int cur = b;
                    window_enter(A.win, cur, on, b, target);
                    if (!on) won = 0;
                }
                if (st >= 0) {
                    // the previous item of the ciphertext must have finished (a
                    // pool ciphertext's: on any CTA)
                    const volatile int *dk = pool ? A.pool_done + k : done + k;
                    unsigned polls = 0;
                    while (*dk != prev) {
                        if (++polls > A.wait_limit) {
                            atomicOr(A.status, kStatusWaitLimit);
                            st = -1;
                            break;
                        }
                        __nanosleep(32);
                    }
                    if (pool) __threadfence();
                    else __threadfence_block();
                }
                plan[wk][0] = st;
                plan[wk][1] = k;
                plan[wk][2] = pool;
            }
            group_sync(bar, kT64);
            {
                const int st = plan[wk][0], k = plan[wk][1], pool = plan[wk][2];
                if (st < 0) break;
                const uint32_t r = pool ? A.pool_res[(size_t)k * S + st] : res[k * S + st];
                const uint64_t *acc = A.accs + ((pool ? A.pool_first : first) + (size_t)k) * 4096;
                const uint64_t pol = l2_keep_policy();
                for (int e = tid; e < 4096; e += kT64) s.acc[e >> 11][px(e & 2047)] = ld_keep64(acc + e, pol);
                group_sync(bar, kT64);
                step64<true, true>(s, A.btkey + ((size_t)st * A.Br + r) * rgsw_pairs, A.DG, A.bg_bits, tw, itw, c,
                       A.derive_last ? acc : nullptr, tid, bar, A.digit_tables ? &dt : nullptr);
            }
            // the item again from the plan (not held in registers across the step;
            // the plan changes only after the barrier below)
            const volatile int *pv = plan[wk];
            const int st = pv[0], k = pv[1], pool = pv[2];
            const size_t gid = (pool ? A.pool_first : first) + (size_t)k;
            uint64_t *acc = A.accs + gid * 4096;
            {
                const uint64_t pol = l2_keep_policy();
                for (int e = tid; e < 4096; e += kT64) st_keep64(acc + e, s.acc[e >> 11][px(e & 2047)], pol);
            }
            if (pool) __threadfence();
            group_sync(bar, kT64);
            if (tid == 0) {
                if (pool) {
                    atomicExch(A.pool_done + k, st);
                } else {
                    __threadfence_block();
                    done[k] = st;
                }
            }
            // a pool ciphertext's output right after its last step
            if (pool && st == A.pool_last[k]) br64_output<true>(A, c, itw, gid, s.acc[0], s.acc[1], tid, bar);
        }
        __syncthreads();
        // output, one ciphertext per worker
        for (int k = wk; k < m; k += W) br64_output<true>(A, c, itw, first + (size_t)k, s.acc[0], s.acc[1], tid, bar);
        __syncthreads();
    }
    // a CTA counts into every bucket it has not counted into yet
    if (threadIdx.x == 0 && A.win.count) {
        const int old = atomicMax(&wcur, A.win.buckets);
        for (int x = old; x < A.win.buckets; x++) atomicAdd(A.win.count + x, 1u);
    }
}

// Extraction of canonical NTT RLWEs (u64) for the key-switch entry point.
__global__ void __launch_bounds__(kT64) extract64_kernel(const uint64_t *__restrict__ rlwe, size_t count,
                                                        uint64_t *__restrict__ extract,
                                                        const ulonglong2 *__restrict__ itw,
                                                        const __grid_constant__ Ntt64Consts c)
{
    __shared__ uint64_t buf[2][2048];
    const int tid = threadIdx.x;
    for (size_t ci = blockIdx.x; ci < count; ci += gridDim.x) {
        const uint64_t *in = rlwe + ci * 4096;
        for (int e = tid; e < 2048; e += kT64) {
            buf[0][e] = in[2047 - e];
            buf[1][e] = in[2048 + e];
        }
        __syncthreads();
        ntt64_inv_2048<128, false>(buf[tid >> 7], itw, c, tid & 127, 1 + (tid >> 7));
        __syncthreads();
        uint64_t *ext = extract + ci * kExtract64;
        for (int e = tid; e < 2048; e += kT64) ext[e] = buf[0][e];
        if (tid == 0) ext[2048] = buf[1][0];
        __syncthreads();
    }
}

struct Ks64Args {
    const uint64_t *ext;
    size_t count;
    const uint64_t *kskey;   // [(d*digitKS + j)*N + i][ks_row]
    uint64_t *out;
    const uint32_t *out_idx;   // optional: ciphertext ci is written to out + out_idx[ci] * (n+1)
    int n, N, digitKS;
    uint32_t Bks, ks_row, q, modswitch;
    int fold;   // rows between mod-Q folds of the 64-bit sums, a multiple of 8
    uint64_t Q;
};

__device__ __forceinline__ uint64_t scale_round64(uint64_t x, uint64_t new_mod, uint64_t old_mod)
{
    const unsigned __int128 num = (unsigned __int128)old_mod + 2 * (unsigned __int128)x * new_mod;
    return (uint64_t)(num / (2 * (unsigned __int128)old_mod));
}

// LWE_keyswitch (LWE.cpp:233-253) + optional LWE_modswitch, one CTA per
// ciphertext; 64-bit sums are folded mod Q every 256 rows (256 Q < 2^64).
// One CTA per ciphertext, one thread per two words of a key row (ks_row / 2
// threads, one 128-bit load per row), eight rows in flight per iteration;
// the 64-bit sums are folded mod Q every A.fold rows (fold * Q < 2^64).
constexpr int kKs64Unroll = 8;

__global__ void __launch_bounds__(512) lwe_ks64_kernel(const __grid_constant__ Ks64Args A)
{
    extern __shared__ uint8_t digits[];   // [N][digitKS]
    const int n = A.n, N = A.N, D = A.digitKS, t = threadIdx.x;
    const uint64_t Q = A.Q;
    const size_t rs2 = A.ks_row / 2;
    const ulonglong2 *key2 = reinterpret_cast<const ulonglong2 *>(A.kskey);
    for (size_t ci = blockIdx.x; ci < A.count; ci += gridDim.x) {
        const uint64_t *ext = A.ext + ci * kExtract64;
        for (int i = t; i < N; i += blockDim.x) {
            uint64_t a = ext[i];
            for (int j = 0; j < D; j++) {
                digits[i * D + j] = (uint8_t)(a % A.Bks);
                a /= A.Bks;
            }
        }
        __syncthreads();
        uint64_t s0 = 0, s1 = 0;
        const int total = N * D;
        int i = 0, j = 0, rows = 0;
        for (int r0 = 0; r0 < total; r0 += kKs64Unroll) {
            ulonglong2 v[kKs64Unroll];
#pragma unroll
            for (int u = 0; u < kKs64Unroll; u++) {
                v[u] = make_ulonglong2(0, 0);
                if (r0 + u < total) {
                    const uint32_t d = digits[r0 + u];
                    v[u] = __ldg(key2 + ((size_t)(d * D + j) * N + i) * rs2 + t);
                }
                if (++j == D) {
                    j = 0;
                    ++i;
                }
            }
#pragma unroll
            for (int u = 0; u < kKs64Unroll; u++) {
                s0 += v[u].x;
                s1 += v[u].y;
            }
            rows += kKs64Unroll;
            if (rows >= A.fold) {
                rows = 0;
                s0 %= Q;
                s1 %= Q;
            }
        }
        const uint64_t b0 = ext[N];
        const uint64_t Q8 = Q / 8 + 1;
        uint64_t *out = A.out + (A.out_idx ? (size_t)A.out_idx[ci] : ci) * (size_t)(n + 1);
        const uint64_t sums[2] = {s0, s1};
#pragma unroll
        for (int c2 = 0; c2 < 2; c2++) {
            const int k = 2 * t + c2;
            if (k <= n) {
                const uint64_t sred = sums[c2] % Q;
                uint64_t v;
                if (k < n) v = sred ? Q - sred : 0;
                else v = ((b0 + Q8) % Q + Q - sred) % Q;
                out[k] = A.modswitch ? scale_round64(v, A.q, Q) : v;
            }
        }
        __syncthreads();
    }
}

// Split form for a few ciphertexts (a lone gate's key switch would otherwise
// run on one CTA): CTA (ci, slice) sums rows [slice * per, ...) of
// ciphertext ci (per <= fold rows, so its 64-bit sums cannot overflow),
// reduces them mod Q and adds them into part[ci][ks_row] (zeroed before;
// slices * Q < 2^64); ks64_final_kernel reduces and writes the outputs.
__global__ void __launch_bounds__(512) ks64_partial_kernel(const __grid_constant__ Ks64Args A,
                                                           unsigned long long *part, int slices)
{
    const int N = A.N, D = A.digitKS, t = threadIdx.x;
    const uint64_t Q = A.Q;
    const size_t rs2 = A.ks_row / 2;
    const ulonglong2 *key2 = reinterpret_cast<const ulonglong2 *>(A.kskey);
    const int total = N * D, per = (total + slices - 1) / slices;
    const size_t ci = blockIdx.x / slices;
    const int r0 = (int)(blockIdx.x % slices) * per, r1 = min(total, r0 + per);
    if (ci >= A.count) return;
    const uint64_t *ext = A.ext + ci * kExtract64;
    uint64_t s0 = 0, s1 = 0;
    for (int r = r0; r < r1; r++) {
        const int i = r / D, j = r - i * D;
        uint64_t a = ext[i];
        for (int jj = 0; jj < j; jj++) a /= A.Bks;
        const uint32_t d = (uint32_t)(a % A.Bks);
        const ulonglong2 v = __ldg(key2 + ((size_t)(d * D + j) * N + i) * rs2 + t);
        s0 += v.x;
        s1 += v.y;
    }
    unsigned long long *p = part + ci * A.ks_row + 2 * (size_t)t;
    atomicAdd(p + 0, (unsigned long long)(s0 % Q));
    atomicAdd(p + 1, (unsigned long long)(s1 % Q));
}

__global__ void ks64_final_kernel(const __grid_constant__ Ks64Args A, const unsigned long long *part)
{
    const uint64_t Q = A.Q, Q8 = Q / 8 + 1;
    const size_t w = (size_t)A.n + 1;
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < A.count * w; x += (size_t)gridDim.x * blockDim.x) {
        const size_t ci = x / w;
        const int k = (int)(x - ci * w);
        const uint64_t sm = part[ci * A.ks_row + k] % Q;
        uint64_t v;
        if (k < A.n) v = sm ? Q - sm : 0;
        else v = ((A.ext[ci * kExtract64 + A.N] + Q8) % Q + Q - sm) % Q;
        A.out[(A.out_idx ? (size_t)A.out_idx[ci] : ci) * w + k] = A.modswitch ? scale_round64(v, A.q, Q) : v;
    }
}

}  // namespace dev

static int sms_of(Context &c)
{
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, c.device);
    return v > 0 ? v : 1;
}

int launch_derive_keys64(Context &c, uint64_t *d_keys, size_t count, const ulonglong2 *d_cf, cudaStream_t st)
{
    if (!count) return FHEACC_OK;
    dev::derive_keys64_kernel<<<(unsigned)std::min<size_t>((count * 4 * c.p.N + 255) / 256, 8192), 256, 0, st>>>(
        d_keys, count, (int)c.p.digitG, c.p.N, d_cf, c.p.Q);
    c.launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "derive keys launch");
}

int launch_shoup_pairs64(Context &c, const uint64_t *d_in, ulonglong2 *d_out, size_t n, cudaStream_t st)
{
    if (!n) return FHEACC_OK;
    unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, (size_t)sms_of(c) * 32);
    dev::shoup_pairs64_kernel<<<blocks, 256, 0, st>>>(d_in, d_out, n, c.p.Q);
    c.launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "shoup pairs launch");
}

int launch_ntt64(Context &c, uint64_t *d_polys, size_t count, bool inverse, cudaStream_t st)
{
    if (!count) return FHEACC_OK;
    size_t blocks = std::min<size_t>((count + 1) / 2, (size_t)sms_of(c) * 8);
    if (inverse) {
        dev::ntt64_kernel<true><<<(unsigned)blocks, dev::kT64, 0, st>>>(d_polys, count, c.d_itw64, c.nc64);
        c.launches++;
    } else {
        dev::ntt64_kernel<false><<<(unsigned)blocks, dev::kT64, 0, st>>>(d_polys, count, c.d_tw64, c.nc64);
        c.launches++;
    }
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "ntt64 launch");
}

int launch_rlwe_mult_rgsw64(Context &c, const uint64_t *d_acc, const uint64_t *d_rgsw, uint64_t *d_out,
                            size_t count, size_t stride, cudaStream_t st)
{
    if (!count) return FHEACC_OK;
    const size_t rw = (size_t)c.p.digitG * 4 * 2048;
    if (stride != 0 && stride != rw) return c.fail(FHEACC_EINVAL, "RGSW stride: 0 or one RGSW");
    const size_t words = (stride ? count : 1) * rw;
    // Shoup pairs of the RGSWs, after the last-digit identity when it applies
    // (2 of the 2 digitG digit NTTs of a product saved); a call of a few
    // products keeps the plain RGSWs, whose derivation would cost it more
    // (PSI query: homo_expand 7.87 -> 7.51 ms, its 1-item CMUXes 0.79 -> 0.90 ms)
    // a call of at most two CTAs per SM of (product, digit) pairs splits each
    // product over its digits, for latency (PSI query: the 11 one-RLWE CMUXes of
    // its blind rotation 0.84 -> 0.48 ms, the 7-level CMUX tree 0.53 -> 0.33 ms)
    const size_t DG = c.p.digitG;
    const bool split = count * DG <= (size_t)sms_of(c) * 2 && (uint64_t)DG * 4 < UINT64_MAX / c.p.Q;
    const bool derive = !split && c.dp.last_digit_from_acc && c.d_cf64 && count >= 16;
    const size_t partial_words = split ? count * DG * 4096 : 0;
    int rc = ensure_scratch(c, c.io, words * (sizeof(ulonglong2) + (derive ? sizeof(uint64_t) : 0)) +
                                         partial_words * sizeof(uint64_t));
    if (rc) return rc;
    ulonglong2 *pairs = (ulonglong2 *)c.io.ptr;
    const uint64_t *src = d_rgsw;
    if (derive) {
        uint64_t *staged = reinterpret_cast<uint64_t *>(pairs + words);
        cudaError_t e = cudaMemcpyAsync(staged, d_rgsw, words * sizeof(uint64_t), cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return c.cuda_fail(e, "RGSW staging");
        rc = launch_derive_keys64(c, staged, words / rw, c.d_cf64, st);
        if (rc) return rc;
        src = staged;
    }
    rc = launch_shoup_pairs64(c, src, pairs, words, st);
    if (rc) return rc;
    if (split) {
        uint64_t *partial = reinterpret_cast<uint64_t *>(pairs + words);
        const size_t smem = sizeof(dev::Step64SmemT<false>);
        cudaFuncSetAttribute(dev::rlwe_mult_rgsw64_split_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        dev::rlwe_mult_rgsw64_split_kernel<<<(unsigned)(count * DG), dev::kT64, smem, st>>>(
            d_acc, pairs, partial, stride, (int)DG, c.p.BG_bits, c.d_tw64, c.d_itw64, c.nc64);
        c.launches++;
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return c.cuda_fail(e, "rlwe_mult_rgsw64 split launch");
        const unsigned blocks = (unsigned)std::min<size_t>((count * 4096 + 255) / 256, (size_t)sms_of(c) * 4);
        dev::rlwe_split_sum64_kernel<<<blocks, 256, 0, st>>>(partial, d_out, count, (int)DG, c.nc64);
        c.launches++;
        e = cudaGetLastError();
        return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "rlwe_mult_rgsw64 split sum launch");
    }
    // no digit tables here: their 20 KB of shared memory cost this kernel more
    // L1 (twiddles, the shared RGSW) than they saved (homo_expand 7.9 -> 8.4 ms)
    const size_t smem = sizeof(dev::Step64SmemT<false>);
    cudaFuncSetAttribute(dev::rlwe_mult_rgsw64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    size_t blocks = std::min<size_t>(count, (size_t)sms_of(c) * 2);
    dev::rlwe_mult_rgsw64_kernel<<<(unsigned)blocks, dev::kT64, smem, st>>>(
        d_acc, pairs, d_out, count, stride, (int)c.p.digitG, c.p.BG_bits, c.d_tw64, c.d_itw64, c.nc64, derive ? 1 : 0);
    c.launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "rlwe_mult_rgsw64 launch");
}

int launch_blind_rotate64(Context &c, const uint64_t *d_c1, const uint64_t *d_c2, const int32_t *d_gates,
                          size_t count, uint32_t flags, uint64_t *d_acc_out, uint64_t *d_extract, int max_ctas,
                          cudaStream_t st)
{
    if (!count) return FHEACC_OK;
    if (!c.d_btkey64) return c.fail(FHEACC_ENOKEY, "bootstrap key not uploaded");
    int rc = ensure_scratch(c, c.accs, bootstrap_accs_bytes(c, count));
    if (rc) return rc;
    return launch_blind_rotate64_with(c, d_c1, d_c2, d_gates, count, flags, (uint64_t *)c.accs.ptr, d_acc_out,
                                      d_extract, max_ctas, st);
}

template <int W, int MINB>
static int launch_br64_shape(Context &c, dev::Br64Args A, int max_ctas, cudaStream_t st)
{
    auto kern = dev::br64_kernel<W, MINB>;
    const size_t steps = (size_t)c.p.n * c.p.digitR;
    // group cap: kMaxGroup64 (or the tuned cap) per worker, within the shared memory of one CTA
    int cap = W * (c.tune.br_group > 0 ? std::min(c.tune.br_group, dev::kMaxGroup64) : dev::kMaxGroup64);
    // digit tables when the gadget base allows and shared memory holds them
    // beside a group of at least kMaxGroup64 per worker (else the group first)
    const size_t tbytes = 40 * ((size_t)1 << c.p.BG_bits);
    A.digit_tables = (1 << c.p.BG_bits) <= dev::kMaxTableBG64 &&
                     W * sizeof(dev::Step64SmemT<true>) + 32 + tbytes + (size_t)cap * steps <= kPipeSmemBudget;
    const size_t fixed = W * sizeof(dev::Step64SmemT<true>) + 32 + (A.digit_tables ? tbytes : 0);
    if (fixed + (size_t)cap * steps > kPipeSmemBudget)
        cap = fixed < kPipeSmemBudget ? (int)((kPipeSmemBudget - fixed) / steps) : 0;
    if (cap < 1) return c.fail(FHEACC_EINVAL, "n * digitR too large for the blind rotation's residue table");
    auto smem_of = [&](int group) {
        return W * sizeof(dev::Step64SmemT<true>) + ((size_t)group * steps + 15) / 16 * 16 + (A.digit_tables ? tbytes : 0);
    };
    size_t smem = smem_of(cap);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return c.cuda_fail(e, "br64 smem attribute");
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, W * dev::kT64, smem);
    if (per_sm < 1) per_sm = 1;
    if (c.tune.br_ctas_per_sm > 0) per_sm = std::min(per_sm, c.tune.br_ctas_per_sm);
    size_t blocks = std::min<size_t>((size_t)sms_of(c) * per_sm, (A.count + W - 1) / W);
    if (max_ctas > 0) blocks = std::min<size_t>(blocks, (size_t)max_ctas);
    blocks = std::max<size_t>(blocks, 1);
    // equal claims: the fewest rounds of at most `cap` ciphertexts per CTA
    const size_t rounds = (A.count + blocks * cap - 1) / (blocks * cap);
    A.group = (int)((A.count + blocks * rounds - 1) / (blocks * rounds));
    A.claim_limit = A.count;
    // claim counters after the accumulators, then the remainder pool's state
    A.claim_next = reinterpret_cast<unsigned long long *>(A.accs + A.count * 4096);
    A.pool_cursor = A.claim_next + 1;
    A.pool_done = reinterpret_cast<int *>(A.claim_next + kClaimWords / 2);
    A.pool_last = A.pool_done + kPool64;
    A.pool_res = reinterpret_cast<uint8_t *>(A.pool_last + kPool64);
    // One round of claims whose CTAs would not all take the same number of
    // ciphertexts: each takes count / blocks of its own, and the remainder is
    // shared by all CTAs item by item (a whole ciphertext more on some CTAs
    // would hold the launch for its steps: 2048 gates on 152 CTAs, 14 against
    // a mean of 13.5)
    if (rounds == 1 && c.tune.br_pool != 0 && A.count > blocks && A.count % blocks != 0 &&
        A.count % blocks <= kPool64) {
        A.group = (int)(A.count / blocks);
        A.claim_limit = (size_t)A.group * blocks;
        A.pool_first = A.claim_limit;
        A.pool_count = (int)(A.count - A.claim_limit);
    }
    smem = smem_of(A.group);
    e = cudaMemsetAsync(A.claim_next, 0, kClaimWords * sizeof(uint32_t), st);
    if (e != cudaSuccess) return c.cuda_fail(e, "br64 claim reset");
    if (A.pool_count) {
        dev::br64_pool_init_kernel<<<(unsigned)A.pool_count, dev::kT64, 0, st>>>(A, c.d_tw64, c.d_itw64, c.nc64);
        c.launches++;
        e = cudaGetLastError();
        if (e != cudaSuccess) return c.cuda_fail(e, "br64 pool launch");
    }
    // the window's per-bucket targets assume one round of claims, and its
    // counters are the context's own (A.win.steps < 0: a launch that may run
    // beside another of the same context takes none)
    const bool window_ok = A.win.steps >= 0;
    A.win = dev::StepWindow{};
    int rc = rounds == 1 && window_ok ? prepare_window(c, (int)steps, st, A.win) : FHEACC_OK;
    if (rc) return rc;
    // CTAs that wait on other CTAs (the remainder pool's done words, the step
    // window) need the whole grid resident: a cooperative launch, which fails
    // instead of starting a grid that cannot be co-resident (the grid is sized
    // from the occupancy calculator, so it fits on an idle GPU)
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)blocks);
    cfg.blockDim = dim3(W * dev::kT64);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = (A.pool_count || A.win.count) ? 1 : 0;
    e = cudaLaunchKernelEx(&cfg, kern, A, (const ulonglong2 *)c.d_tw64, (const ulonglong2 *)c.d_itw64, c.nc64);
    c.launches++;
    if (e == cudaSuccess) e = cudaGetLastError();
    return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "br64 launch");
}

int launch_blind_rotate64_with(Context &c, const uint64_t *d_c1, const uint64_t *d_c2, const int32_t *d_gates,
                               size_t count, uint32_t flags, uint64_t *accs, uint64_t *d_acc_out,
                               uint64_t *d_extract, int max_ctas, cudaStream_t st)
{
    return launch_blind_rotate64_indexed(c, d_c1, d_c2, nullptr, nullptr, d_gates, count, flags, accs, d_acc_out,
                                         d_extract, max_ctas, true, st);
}

int launch_blind_rotate64_indexed(Context &c, const uint64_t *d_c1, const uint64_t *d_c2, const uint32_t *d_idx1,
                                  const uint32_t *d_idx2, const int32_t *d_gates, size_t count, uint32_t flags,
                                  uint64_t *accs, uint64_t *d_acc_out, uint64_t *d_extract, int max_ctas,
                                  bool window, cudaStream_t st)
{
    if (!count) return FHEACC_OK;
    if (!c.d_btkey64) return c.fail(FHEACC_ENOKEY, "bootstrap key not uploaded");
    dev::Br64Args A{};
    A.c1 = d_c1; A.c2 = d_c2; A.idx1 = d_idx1; A.idx2 = d_idx2; A.gates = d_gates; A.count = count;
    A.win.steps = window ? 0 : -1;
    A.btkey = c.d_btkey64; A.accs = accs; A.acc_out = d_acc_out; A.extract = d_extract;
    A.n = c.p.n; A.DG = (int)c.p.digitG; A.q = c.p.q; A.embed = c.dp.embed; A.Br = c.p.Br; A.digitR = c.p.digitR;
    A.bg_bits = c.p.BG_bits; A.flags = flags; A.derive_last = (int)c.dp.last_digit_from_acc;
    A.status = c.d_status;
    A.wait_limit = c.tune.debug_wait_limit >= 0 ? (unsigned)c.tune.debug_wait_limit : dev::kWorkerWaitLimit;
    for (int i = 0; i < 8; i++) A.gate_constant[i] = c.dp.gate_constant[i];
    // workers per CTA, by default from the gates per SM (one GB300): up to 1
    // one worker per CTA (3 CTAs per SM), beyond that two, whose shared memory
    // leaves room for the digit tables that three workers' does not (2048
    // gates: 658 ms with two workers and tables, 698 ms with three; 700 gates:
    // 240 ms either way; 304 gates: 98 / 109 / 146 ms with 2 / 1 / 3)
    const size_t sms = (size_t)sms_of(c);
    const int w = c.tune.br_pipes > 0 ? c.tune.br_pipes : count <= sms ? 1 : 2;
    if (w == 3) return launch_br64_shape<3, 1>(c, A, max_ctas, st);
    if (w == 2) return launch_br64_shape<2, 1>(c, A, max_ctas, st);
    return launch_br64_shape<1, 3>(c, A, max_ctas, st);
}

int launch_extract64(Context &c, const uint64_t *d_rlwe, size_t count, uint64_t *d_extract, cudaStream_t st)
{
    if (!count) return FHEACC_OK;
    size_t blocks = std::min<size_t>(count, (size_t)sms_of(c) * 4);
    dev::extract64_kernel<<<(unsigned)blocks, dev::kT64, 0, st>>>(d_rlwe, count, d_extract, c.d_itw64, c.nc64);
    c.launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "extract64 launch");
}

int launch_lwe_keyswitch64(Context &c, const uint64_t *d_extract, size_t count, bool modswitch, uint64_t *d_out,
                           cudaStream_t st, const uint32_t *d_out_idx, void *d_scratch, size_t scratch_bytes)
{
    if (!count) return FHEACC_OK;
    if (!c.d_kskey64) return c.fail(FHEACC_ENOKEY, "LWE key-switch key not uploaded");
    if (c.dp.ks_row > 1024) return c.fail(FHEACC_EINVAL, "n too large for key switch");
    dev::Ks64Args A{};
    A.ext = d_extract; A.count = count; A.kskey = c.d_kskey64; A.out = d_out; A.out_idx = d_out_idx;
    A.n = c.p.n; A.N = c.p.N; A.digitKS = (int)c.p.digitKS; A.Bks = c.p.Bks; A.ks_row = c.dp.ks_row;
    A.q = c.p.q; A.modswitch = modswitch ? 1u : 0u; A.Q = c.p.Q;
    // key words are < Q: (fold + 1) Q must stay below 2^64
    const uint64_t fold = std::min<uint64_t>(256, UINT64_MAX / c.p.Q - 1);
    A.fold = (int)std::max<uint64_t>(8, fold & ~(uint64_t)7);
    const unsigned threads = c.dp.ks_row / 2;   // ks_row: a multiple of 32 words, > n
    const size_t sms = (size_t)sms_of(c);
    // from two gates per SM: the tiled form (lwe_ks.cu), each row group read
    // from L2 once per gate block
    if (d_scratch && ks64_tiled_applies(c, count, (int)sms, scratch_bytes))
        return launch_ks64_tiled(c, d_extract, count, modswitch, d_out, d_out_idx, d_scratch, (int)sms, st);
    // a few ciphertexts: each one's rows split over many CTAs, with at most
    // `fold` rows per CTA and slices * Q < 2^64
    const int rows = c.p.N * (int)c.p.digitKS;
    const size_t max_slices = std::min<uint64_t>(UINT64_MAX / c.p.Q, 4096);
    const size_t slices = std::min<size_t>(max_slices, std::max<size_t>((size_t)(rows + A.fold - 1) / A.fold,
                                                                         sms * 8 / std::max<size_t>(count, 1)));
    if (d_scratch && count < 2 * sms && count * c.dp.ks_row * sizeof(uint64_t) <= scratch_bytes &&
        (size_t)(rows + slices - 1) / slices <= (size_t)A.fold) {
        unsigned long long *part = reinterpret_cast<unsigned long long *>(d_scratch);
        cudaError_t e = cudaMemsetAsync(part, 0, count * c.dp.ks_row * sizeof(uint64_t), st);
        if (e != cudaSuccess) return c.cuda_fail(e, "key switch partials reset");
        dev::ks64_partial_kernel<<<(unsigned)(count * slices), threads, 0, st>>>(A, part, (int)slices);
        c.launches++;
        e = cudaGetLastError();
        if (e != cudaSuccess) return c.cuda_fail(e, "key switch partial launch");
        const size_t words = count * ((size_t)c.p.n + 1);
        dev::ks64_final_kernel<<<(unsigned)std::min<size_t>((words + 255) / 256, 1024), 256, 0, st>>>(A, part);
        c.launches++;
        e = cudaGetLastError();
        return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "key switch final launch");
    }
    const size_t smem = (size_t)c.p.N * c.p.digitKS;
    size_t blocks = std::min<size_t>(count, sms * 6);
    dev::lwe_ks64_kernel<<<(unsigned)blocks, threads, smem, st>>>(A);
    c.launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "lwe_ks64 launch");
}

}  // namespace fheacc
