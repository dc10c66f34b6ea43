// blind_rotate32.cu -- batched blind rotation of FHEW/AP gate bootstrapping,
// N = 1024, Q < 2^27 (32-bit words).
//
// Reference behaviour: the accumulate loop of RLWE::eval_bootstrap
// (FHE_ACC_runtime/src/RLWE.cpp:733-767) -- LWE_evaluate (LWE.cpp:203-222),
// acc_initialization (RLWE.cpp:706-724), then for every LWE coefficient i and
// refresh digit j with a non-zero residue r an RLWE_mult_RGSW (RLWE.cpp:642-704)
// with btkey[r][j][i] -- followed by the NTT_a_transpose and inverse NTT that
// open LWE_keyswitch (LWE.cpp:235-238). On the FPGA this loop is the host's
// instruction issue (myfpga.cpp:1446-1492) feeding iNTT_module.sv,
// NTT_leading_stage.sv, poly_mult_RLWE.sv and accumulator.sv.
//
// Schedule. The grid is persistent; each CTA claims a group of consecutive
// ciphertexts from a counter (the launcher fits the group size to the batch:
// the fewest rounds of at most kMaxGroup per pipeline, or the tuned cap) and claims again
// until the batch is done. Steps are the OUTER loop: a CTA applies step s to every ciphertext of
// its group before step s + 1, so the CTAs walk through the bootstrapping key
// together and the 23 RGSW keys of a step (1.5 MB) are mostly served from L2.
// Accumulators live in global memory (8 KB per ciphertext, L2-resident for
// batches of thousands).
//
// Inside a CTA the (step, ciphertext) items flow through a two-stage warp-
// specialised pipeline, one item per period, periods separated by
// __syncthreads:
//   inverse-NTT warps (2): load acc of item k+1, inverse NTT of a and b,
//                          canonical time-domain coefficients -> tslot[k+1 & 1]
//   digit warps (2*(digitG-1)): item k: digit h < digitG-1 of poly p from
//                          tslot[k & 1], forward NTT (first two stages by
//                          table lookup when BG <= kMaxTableBG,
//                          ntt_fwd_1024_digit) -> dbuf
//   all warps, after __syncthreads: multiply-accumulate item k with its RGSW
//                          key (64-bit sums, one Montgomery reduction per
//                          output) -> acc (global)
// An item whose ciphertext is still in the digit stage waits one period.
//
// Last digit. Parameter validation requires Q < BG^digitG, so the digits
// recompose each canonical coefficient exactly, so sum_h BG^h NTT(digit_h) equals the NTT-domain
// accumulator. The keys are uploaded with that identity folded in
// (DevParams::last_digit_from_acc), the warps of the last digit skip their
// transform, and the MAC multiplies the accumulator (read from global memory
// before it is overwritten) by the last key row: 2 of the 2*digitG digit NTTs
// of a step are saved, with results unchanged mod Q.
//
// Scaling. The bootstrap key is uploaded times 2^32 N^-1 mod Q: the Montgomery
// reduction of the sums removes the 2^32, and the N^-1 the reference's iNTT
// applies is already in the accumulator, so the inverse transforms skip it
// (ntt_inv_1024_noscale). The initial accumulator is the reference's test
// vector times N^-1; canonical NTT-domain accumulators are multiplied by N on
// the way out. All results are the reference's values mod Q.
//
// Global layouts. Accumulators and bootstrap-key polys are stored "B-tiled":
// element 32 l + r of a poly sits at word ((r / 4) * 32 + l) * 4 + r % 4, so a
// warp loading a poly into the NTT's contiguous register layout, and the MAC
// threads reading keys and writing accumulators, move 512 contiguous bytes
// per instruction.
#include "ctx.hpp"
#include "step32.cuh"
#include <algorithm>

namespace fheacc {
namespace dev {

constexpr int kMaxGroup = 24;   // ciphertexts per pipeline and claim (residue table in shared memory)
constexpr int kMaxTableBG = 512;   // largest gadget base with digit tables (20 BG bytes of shared memory)

struct PipeArgs {
    const uint64_t *c1, *c2;
    const uint32_t *idx1, *idx2;   // optional: gate g reads c1 + idx1[g] * (n+1) (else g)
    const int32_t *gates;
    size_t count;
    const uint32_t *btkey;   // B-tiled polys, [(i*digitR + j)*Br + r][digitG][2][2][1024]
    uint32_t *accs;          // scratch [count][2][1024], B-tiled, values < 2Q
    uint64_t *acc_out;       // optional: canonical NTT accumulators [count][2048]
    uint32_t *extract;       // optional: [count][kExtractStride]
    int group;               // ciphertexts per claim (<= kMaxGroup per pipeline)
    int n;
    uint32_t q, embed, Br, digitR, bg_bits, flags;
    uint32_t qinv_neg;         // -Q^-1 mod 2^32 (keys carry 2^32 N^-1, see DevParams::key_factor)
    uint32_t tv_pos, tv_neg;   // test-vector values +-(Q/8 + 1) times N^-1
    uint32_t nmul, nmuls;      // N mod Q and its Shoup companion (canonical accumulators out)
    uint32_t w21, w31;         // rou[2] rou[1], rou[3] rou[1] mod Q (digit tables)
    uint32_t derive_last;      // last digit's NTT from the accumulator (DevParams::last_digit_from_acc)
    uint32_t digit_tables;     // first two digit-NTT stages by table lookup (BG <= kMaxTableBG)
    uint64_t gate_constant[8];
    unsigned long long *claim_next;   // next unclaimed ciphertext (zeroed before the launch)
    unsigned *status;                 // set to kStatusWaitLimit if a pipeline gave up waiting
    int idle_limit;                   // idle periods before such a wait gives up (kIdleLimit)
};

// Periods a pipeline idles with a claimed item whose ciphertext's previous step
// another pipeline still holds, before it gives up and flags the launch.
constexpr int kIdleLimit = 1 << 22;

// Shared memory of one CTA. tslot holds lane-major copies of the inverse-NTT
// warps' registers (layout A), dbuf the digit NTT outputs as swizzled rows
// (layout B); both double as the per-warp transpose scratch.
template <int NB>
struct PipeSmem {
    uint32_t tslot[2][2][kN32];   // time-domain accumulators, one slot per pipeline stage
    uint32_t dbuf[NB][kN32];      // digit NTT outputs / transposes of the digit warps
    int ctl[2][16];               // the pipeline's plans, one per period parity (pipe_plan)
};

// Bytes of dynamic shared memory before the digit tables: one PipeSmem per
// pipeline, then the residue table [group][n * digitR], rounded up to 16.
template <int NB, int NP>
__host__ __device__ constexpr size_t pipe_tables_offset(int group, size_t steps)
{
    return NP * sizeof(PipeSmem<NB>) + ((size_t)group * steps + 15) / 16 * 16;
}

__device__ __forceinline__ void load_btile(uint32_t (&x)[32], const uint32_t *src, int lane)
{
    const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
#pragma unroll
    for (int qq = 0; qq < 8; qq++) {
        const uint4 v = __ldcg(s4 + qq * 32 + lane);
        x[4 * qq] = v.x; x[4 * qq + 1] = v.y; x[4 * qq + 2] = v.z; x[4 * qq + 3] = v.w;
    }
}

// Layout-B registers of the poly reversed in index (NTT_a_transpose).
__device__ __forceinline__ void load_btile_reversed(uint32_t (&x)[32], const uint32_t *src, int lane)
{
    const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
#pragma unroll
    for (int qq = 0; qq < 8; qq++) {
        const uint4 v = __ldcg(s4 + (7 - qq) * 32 + (31 - lane));
        x[4 * qq] = v.w; x[4 * qq + 1] = v.z; x[4 * qq + 2] = v.y; x[4 * qq + 3] = v.x;
    }
}

__device__ __forceinline__ void store_btile(uint32_t *dst, const uint32_t (&x)[32], int lane)
{
    uint4 *d4 = reinterpret_cast<uint4 *>(dst);
#pragma unroll
    for (int qq = 0; qq < 8; qq++) __stcg(d4 + qq * 32 + lane, make_uint4(x[4 * qq], x[4 * qq + 1], x[4 * qq + 2],
                                                                       x[4 * qq + 3]));
}

// load_btile / store_btile of an accumulator that the next step reads again:
// the L2 evict-last policy (l2hint.cuh) keeps it in L2 while the key tiles
// stream through.
__device__ __forceinline__ void load_btile_keep(uint32_t (&x)[32], const uint32_t *src, int lane)
{
    const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
    const uint64_t pol = l2_keep_policy();
#pragma unroll
    for (int qq = 0; qq < 8; qq++) {
        const uint4 v = ld_keep(s4 + qq * 32 + lane, pol);
        x[4 * qq] = v.x; x[4 * qq + 1] = v.y; x[4 * qq + 2] = v.z; x[4 * qq + 3] = v.w;
    }
}

__device__ __forceinline__ void store_btile_keep(uint32_t *dst, const uint32_t (&x)[32], int lane)
{
    uint4 *d4 = reinterpret_cast<uint4 *>(dst);
    const uint64_t pol = l2_keep_policy();
#pragma unroll
    for (int qq = 0; qq < 8; qq++)
        st_keep(d4 + qq * 32 + lane, make_uint4(x[4 * qq], x[4 * qq + 1], x[4 * qq + 2], x[4 * qq + 3]), pol);
}

// Plans period t + 1 of one pipeline (run by one thread of it while the other
// threads multiply-accumulate period t's digit item). C is period t's plan, Nx
// receives the next. The pipelines of a CTA share the group's items: a cursor
// walks the (step, ciphertext) items step-major, and an item is issued only
// once the previous item of its ciphertext (its last earlier step with a
// non-zero residue) has finished, which keeps every ciphertext's steps in the
// reference's order. The digit item of period t finishes before period t + 1
// starts, so an item that follows it may be issued for period t + 1; the
// planning thread marks it finished (done[]) for the other pipelines after
// the MAC barrier.
// Plan: [0, 1] item of the inverse-NTT warps; [2, 3] item of the digit warps
// (ciphertext < 0: none); [4] slot; [5] cursor exhausted; [6] inverse-NTT
// item valid; [7] stop; [8, 9, 10] claimed item waiting to be issued (step < 0:
// none) and the step its ciphertext must have finished; [11] periods idled in
// a row waiting for it. done[k]: last finished step of ciphertext k.
__device__ __noinline__ void pipe_plan(const int *C, int *Nx, volatile int *done, int *cursor, const uint8_t *res,
                                       int m, int S, int mode, unsigned *status, int idle_limit)
{
    // period t's inverse-NTT item moves to the digit warps
    Nx[2] = C[6] ? C[0] : -1;
    Nx[3] = C[6] ? C[1] : -1;
    Nx[5] = C[5];
    Nx[8] = C[8];
    Nx[9] = C[9];
    Nx[10] = C[10];
    if (Nx[8] < 0 && !Nx[5]) {
        for (;;) {
            const int idx = atomicAdd(cursor, 1);
            if (idx >= S * m) {
                Nx[5] = 1;
                break;
            }
            const int st = idx / m, k = idx - st * m;
            if (step_issued(res + k * S, st, mode)) {
                int prev = st - 1;
                while (prev >= 0 && !step_issued(res + k * S, prev, mode)) prev--;
                Nx[8] = st;
                Nx[9] = k;
                Nx[10] = prev;
                break;
            }
        }
    }
    const bool hv = Nx[8] >= 0 && (done[Nx[9]] == Nx[10] || (Nx[9] == C[3] && Nx[10] == C[2]));
    if (hv) {
        __threadfence_block();
        Nx[0] = Nx[8];
        Nx[1] = Nx[9];
        Nx[8] = -1;
    } else {
        Nx[0] = 0;
        Nx[1] = -1;
    }
    // a wait on another pipeline ends within a few periods; one that does not
    // is abandoned (bounded wait) and flagged
    Nx[11] = (!hv && Nx[3] < 0 && Nx[8] >= 0) ? C[11] + 1 : 0;
    if (Nx[11] > idle_limit) {
        atomicOr(status, kStatusWaitLimit);
        Nx[8] = -1;
        Nx[5] = 1;
    }
    Nx[6] = hv;
    Nx[7] = !hv && Nx[8] < 0 && Nx[3] < 0 && Nx[5];
    // slot: the inverse-NTT warps alternate slots every period
    Nx[4] = C[4] ^ 1;
}

__device__ __forceinline__ void pipe_barrier(int id, int threads)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(threads) : "memory");
}

// LWE_evaluate, the residues and acc_initialization of ciphertext gid (one
// warp; res_k: its row of the residue table; buf: the warp's transpose
// scratch). Kept out of line, so that its registers do not shape the
// pipeline loop's allocation.
__device__ __noinline__ void pipe_init_item(const PipeArgs &A, const Ntt32Consts &c, const uint2 *__restrict__ fwd_tw,
                                            uint32_t *buf, uint8_t *res_k, size_t gid, int lane, uint32_t mu32)
{
    const int n = A.n;
    const uint32_t q = A.q, qmask = q - 1;
    const int g = A.gates[gid];
    const bool x2 = (g == 4 || g == 5);
    const uint64_t *c1 = A.c1 + (A.idx1 ? (size_t)A.idx1[gid] : gid) * (size_t)(n + 1);
    const uint64_t *c2 = A.c2 + (A.idx2 ? (size_t)A.idx2[gid] : gid) * (size_t)(n + 1);
    for (int i = lane; i < n; i += 32) {
        const uint64_t v = x2 ? 2 * (c1[i] - c2[i]) : c1[i] + c2[i];
        uint32_t nega = (q - (uint32_t)(v & qmask)) & qmask;
        for (uint32_t j = 0; j < A.digitR; j++) {
            res_k[i * (int)A.digitR + (int)j] = (uint8_t)(nega % A.Br);
            nega /= A.Br;
        }
    }
    const uint64_t vb = x2 ? 2 * (c1[n] - c2[n]) : c1[n] + c2[n];
    const uint32_t bval = (uint32_t)(vb & qmask);
    const uint64_t gc = A.gate_constant[(unsigned)g < 6u ? g : 6];
    const uint32_t b1 = (uint32_t)(gc & qmask), b2 = (b1 + q / 2) & qmask;
    const uint32_t Q8 = A.tv_pos, negQ8 = A.tv_neg;
    uint32_t x[32];
#pragma unroll
    for (int r = 0; r < 32; r++) {
        const uint32_t idx = lane + 32 * r;
        uint32_t v = 0;
        if (idx % A.embed == 0 && idx / A.embed < q / 2) {
            const uint32_t tmp = (bval - idx / A.embed) & qmask;
            if (b1 < b2) v = (tmp >= b1 && tmp < b2) ? negQ8 : Q8;
            else v = (tmp >= b2 && tmp < b1) ? Q8 : negQ8;
        }
        x[r] = v;
    }
    ntt_fwd_1024(x, c, fwd_tw, buf, lane);
#pragma unroll
    for (int r = 0; r < 32; r++) x[r] = reduce32(x[r], mu32, c.Q);
    uint32_t *acc = A.accs + gid * 2048;
    store_btile_keep(acc + 1024, x, lane);
    uint4 *a4 = reinterpret_cast<uint4 *>(acc);
    const uint64_t pol = l2_keep_policy();
#pragma unroll
    for (int qq = 0; qq < 8; qq++) st_keep(a4 + qq * 32 + lane, make_uint4(0, 0, 0, 0), pol);
    __syncwarp();
}

// Output of poly P of ciphertext gid: the canonical NTT accumulator, or the
// extraction for the key switch (NTT_a_transpose and inverse NTT). One warp,
// out of line as pipe_init_item.
__device__ __noinline__ void pipe_out_poly(const PipeArgs &A, const Ntt32Consts &c, const uint2 *__restrict__ inv_tw,
                                           uint32_t *buf, size_t gid, int P, int lane)
{
    const uint32_t *acc = A.accs + gid * 2048 + P * 1024;
    uint32_t x[32];
    if (A.extract) {
        if (P == 0) load_btile_reversed(x, acc, lane);
        else load_btile(x, acc, lane);
        ntt_inv_1024_noscale(x, c, inv_tw, buf, lane);
        uint32_t *ext = A.extract + gid * kExtractStride;
        if (P == 0) {
#pragma unroll
            for (int r = 0; r < 32; r++) ext[lane + 32 * r] = x[r];
        } else if (lane == 0) {
            ext[1024] = x[0];
        }
    } else {
        load_btile(x, acc, lane);
        uint64_t *out = A.acc_out + gid * 2048 + P * 1024 + 32 * lane;
#pragma unroll
        for (int r = 0; r < 32; r++) {
            const uint32_t v = shoup32(x[r], A.nmul, A.nmuls, c.Q);   // times N: the key factor's N^-1 out
            out[r] = min(v, v - c.Q);
        }
    }
}

// NP pipelines per CTA, each of 2 (digitG - 1) digit warps (the last digit's
// NTT comes from the accumulator) and 2 inverse-NTT warps, all of whose warps
// share the MAC; pipeline p synchronises on named barrier 1 + p.
template <int DG, int NP, int MINB>
__global__ void __launch_bounds__(NP * 32 * (2 * (DG - 1) + 2), MINB)
    br32_pipe_kernel(const __grid_constant__ PipeArgs A, const __grid_constant__ Ntt32Consts c,
                     const uint2 *__restrict__ fwd_tw, const uint2 *__restrict__ inv_tw, uint32_t mu32)
{
    constexpr int DT = DG - 1;   // digit NTTs per poly
    constexpr int GW = 2 * DT;   // digit warps
    constexpr int NW = GW + 2;   // plus the two inverse-NTT warps
    constexpr int PT = 32 * NW;  // threads of a pipeline
    extern __shared__ __align__(16) unsigned char smem_raw[];
    PipeSmem<GW> *pipes = reinterpret_cast<PipeSmem<GW> *>(smem_raw);
    uint8_t *res = smem_raw + NP * sizeof(PipeSmem<GW>);   // [group][n * digitR] residues
    __shared__ int done[kMaxGroup * NP];
    __shared__ int cursor;
    __shared__ unsigned long long claim_first;
    __shared__ int claim_m;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int pl = warp / NW, pw = warp - pl * NW;
    PipeSmem<GW> &s = pipes[pl];
    const int S = A.n * (int)A.digitR;
    const size_t rgsw_words = (size_t)DG * 4 * 1024;
    const int mode = issue_mode(A.flags);

    // digit tables (ntt_fwd_1024_digit): t1, t23, t123, each [BG][copies]
    const int cl = digit_table_copies_log2((int)A.bg_bits);
    const int BGC = A.digit_tables ? (1 << A.bg_bits) << cl : 0;
    uint32_t *t1 = reinterpret_cast<uint32_t *>(smem_raw + pipe_tables_offset<GW, NP>(A.group, S));
    uint2 *t23 = reinterpret_cast<uint2 *>(t1 + BGC), *t123 = t23 + BGC;
    for (int i = threadIdx.x; i < BGC; i += blockDim.x) {
        const uint64_t Q = c.Q, y = (uint64_t)(i >> cl);
        t1[i] = (uint32_t)(y * c.fw[1] % Q);
        t23[i] = make_uint2((uint32_t)(y * c.fw[2] % Q), (uint32_t)(y * c.fw[3] % Q));
        t123[i] = make_uint2((uint32_t)(y * A.w21 % Q), (uint32_t)(y * A.w31 % Q));
    }
    const DigitTables dt{t1, t23, t123, cl};
    __syncthreads();

    // each CTA claims A.group consecutive ciphertexts at a time until none are left
    for (;;) {
        if (threadIdx.x == 0) {
            const unsigned long long f = atomicAdd(A.claim_next, (unsigned long long)A.group);
            claim_first = f;
            claim_m = f < A.count ? (int)min((unsigned long long)A.group, (unsigned long long)A.count - f) : 0;
        }
        __syncthreads();
        const size_t first = claim_first;
        const int m = claim_m;
        if (m == 0) break;

        // ---- prologue: LWE_evaluate, residues, acc_initialization (one warp per ciphertext)
        for (int k = warp; k < m; k += NP * NW)
            pipe_init_item(A, c, fwd_tw, pw < GW ? s.dbuf[pw] : s.tslot[0][pw - GW], res + k * S, first + (size_t)k,
                           lane, mu32);
        if (threadIdx.x == 0) cursor = 0;
        for (int k = threadIdx.x; k < m; k += blockDim.x) done[k] = -1;
        if (pw == 0 && lane == 0) {
            int *c0 = s.ctl[1];           // a period before the first: nothing in flight
            c0[0] = 0; c0[1] = -1;        // item of the inverse-NTT warps
            c0[2] = -1; c0[3] = -1;       // item of the digit warps (ciphertext < 0: none)
            c0[4] = 1;                    // slot written by the inverse-NTT warps
            c0[5] = 0;                    // cursor exhausted
            c0[6] = 0; c0[7] = 0;         // inverse-NTT item valid, stop
            c0[8] = -1;                   // no claimed item waiting
            c0[11] = 0;                   // idle periods in a row
        }
        __syncthreads();

        // ---- NP pipelines over the (step, ciphertext) items of the group. One
        // thread of each plans the pipeline's next period after each period
        // and publishes the plan in shared memory.
        if (pw == 0 && lane == 0) pipe_plan(s.ctl[1], s.ctl[0], done, &cursor, res, m, S, mode, A.status, A.idle_limit);
        pipe_barrier(1 + pl, PT);
        for (int t = 0;; t ^= 1) {
            const int *ctl = s.ctl[t];
            if (ctl[7]) break;
            const int sh = ctl[4];
            if (pw >= GW) {
                if (ctl[6]) {
                    const int hp = pw - GW;
                    uint32_t x[32];
                    load_btile_keep(x, A.accs + (first + (size_t)ctl[1]) * 2048 + hp * 1024, lane);
                    uint32_t *ts = s.tslot[sh][hp];
                    ntt_inv_1024_noscale(x, c, inv_tw, ts, lane);
                    store_row(ts, lane, x);
                }
            } else if (ctl[3] >= 0) {
                const int p = pw / DT, h = pw % DT;
                const uint32_t shift = A.bg_bits * h, mask = (1u << A.bg_bits) - 1;
                uint32_t x[32];
                load_row(x, s.tslot[sh ^ 1][p], lane);
#pragma unroll
                for (int r = 0; r < 32; r++) x[r] = (x[r] >> shift) & mask;
                if (A.digit_tables) ntt_fwd_1024_digit(x, c, fwd_tw, s.dbuf[pw], dt, lane);
                else ntt_fwd_1024(x, c, fwd_tw, s.dbuf[pw], lane);
                store_row(s.dbuf[pw], lane, x);
            }
            // all warps of the pipeline multiply-accumulate the digit warps'
            // item once its digit NTTs are in shared memory; one thread first
            // plans the next period
            pipe_barrier(1 + pl, PT);
            if (pw == 0 && lane == 0) pipe_plan(ctl, s.ctl[t ^ 1], done, &cursor, res, m, S, mode, A.status, A.idle_limit);
            if (ctl[3] >= 0) {
                const int gk = ctl[3], gs = ctl[2];
                const uint32_t rr = res[gk * S + gs];
                const uint4 *key = reinterpret_cast<const uint4 *>(A.btkey + ((size_t)gs * A.Br + rr) * rgsw_words);
                uint4 *acc = reinterpret_cast<uint4 *>(A.accs + (first + (size_t)gk) * 2048);
                for (int u = pw * 32 + lane; u < 256; u += PT)
                    mac_chunk<DG, true, true>(u, key, s.dbuf, acc, c.Q, A.qinv_neg, acc);
            }
            pipe_barrier(1 + pl, PT);
            // the digit item is finished: other pipelines may issue its
            // ciphertext's next step
            if (pw == 0 && lane == 0 && ctl[3] >= 0) {
                __threadfence_block();
                done[ctl[3]] = ctl[2];
            }
        }
        __syncthreads();

        // ---- epilogue: NTT accumulators out, or extraction for the key switch
        for (int t = warp; t < 2 * m; t += NP * NW)
            pipe_out_poly(A, c, inv_tw, pw < GW ? s.dbuf[pw] : s.tslot[0][pw - GW], first + (size_t)(t >> 1), t & 1,
                          lane);
        __syncthreads();
    }
}

// ---- Latency form: one ciphertext per CTA, keys prefetched into shared memory.
//
// Below one ciphertext per SM the pipelines above have nothing to overlap: a
// lone ciphertext's steps are a serial chain, and each step waits for its 64 KB
// key from DRAM and for its accumulator's round trip through L2. This kernel
// keeps the accumulator in shared memory and streams the keys of the next two
// issued steps into two shared-memory buffers with bulk asynchronous copies
// (cp.async.bulk, completion counted in bytes on an mbarrier), so a step is
// the three transform phases and nothing else:
//   inverse-NTT warps (2): acc (NTT domain) -> inverse NTT -> tslot
//   digit warps (2 (digitG - 1)): digits of tslot -> digit NTTs -> dbuf
//   all warps: wait for the step's key buffer, multiply-accumulate -> acc
// The arithmetic is the pipelines' (same transforms, same 64-bit sums and
// Montgomery reduction), so the outputs are identical word for word.

// Polls of an mbarrier before a key wait gives up and flags the launch (the
// copy of one key takes microseconds).
constexpr int kSoloWaitLimit = 1 << 22;

// Digit-table copies of the latency form (8 up to BG = 128: the twiddle
// copies take the shared memory of the other 8).
__host__ __device__ constexpr int solo_table_copies_log2(int bg_bits) { return bg_bits <= 7 ? 3 : 0; }

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bulk copy of `bytes` (a multiple of 16, both addresses 16-byte aligned) from
// global to shared memory, counted on `bar`.
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, unsigned bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(__cvta_generic_to_global(src)), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// Waits for phase `parity` of `bar`; false if it did not complete within
// `limit` polls.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, unsigned parity, int limit)
{
    for (int i = 0; i < limit; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Next issued step after step s (S if none).
__device__ __forceinline__ int solo_next_step(const uint8_t *res, int s, int S, int mode)
{
    for (s++; s < S; s++)
        if (step_issued(res, s, mode)) return s;
    return S;
}

// Multiply-accumulate of chunk u (the elements of mac_chunk) from shared
// memory: the key buffer keeps the global B-tiled order, the accumulator and
// the digit NTTs are swizzled rows. Reads both accumulator chunks before
// writing them.
template <int DG>
__device__ __forceinline__ void mac_chunk_solo(int u, const uint4 *key, const uint32_t (*dbuf)[kN32],
                                               uint32_t (*acc)[kN32], uint32_t Q, uint32_t qinv_neg)
{
    constexpr int DT = DG - 1;
    const int pa = sw_chunk(u & 31, u >> 5);
    uint64_t sa[4] = {0, 0, 0, 0}, sb[4] = {0, 0, 0, 0};
#pragma unroll
    for (int qi = 0; qi < 2 * DG; qi++) {
        const int pp = qi / DG, hh = qi % DG;
        const uint4 dv = hh == DG - 1 ? *reinterpret_cast<const uint4 *>(acc[pp] + pa)
                                      : *reinterpret_cast<const uint4 *>(dbuf[pp * DT + hh] + pa);
        const uint4 a4 = key[((hh * 2 + pp) * 2 + 0) * 256 + u];
        const uint4 b4 = key[((hh * 2 + pp) * 2 + 1) * 256 + u];
        sa[0] += (uint64_t)dv.x * a4.x; sb[0] += (uint64_t)dv.x * b4.x;
        sa[1] += (uint64_t)dv.y * a4.y; sb[1] += (uint64_t)dv.y * b4.y;
        sa[2] += (uint64_t)dv.z * a4.z; sb[2] += (uint64_t)dv.z * b4.z;
        sa[3] += (uint64_t)dv.w * a4.w; sb[3] += (uint64_t)dv.w * b4.w;
    }
    *reinterpret_cast<uint4 *>(acc[0] + pa) =
        make_uint4(mont_reduce_2q(sa[0], Q, qinv_neg), mont_reduce_2q(sa[1], Q, qinv_neg),
                   mont_reduce_2q(sa[2], Q, qinv_neg), mont_reduce_2q(sa[3], Q, qinv_neg));
    *reinterpret_cast<uint4 *>(acc[1] + pa) =
        make_uint4(mont_reduce_2q(sb[0], Q, qinv_neg), mont_reduce_2q(sb[1], Q, qinv_neg),
                   mont_reduce_2q(sb[2], Q, qinv_neg), mont_reduce_2q(sb[3], Q, qinv_neg));
}

// Shared memory of a latency-form CTA: two key buffers, then the accumulator,
// the time-domain polys, the digit NTTs, copies of the forward and inverse
// twiddle tables, the digit tables and the residues. The twiddles are copied
// because L1 does not keep them from one step to the next here: read through
// L1, the first forward NTT of a step took 6000 cycles instead of 2300, each
// of its five per-lane-twiddle stages waiting on L2.
template <int DG>
struct SoloLayout {
    static constexpr int GW = 2 * (DG - 1);
    static constexpr size_t key_bytes = (size_t)DG * 4 * kN32 * sizeof(uint32_t);
    static constexpr size_t acc_off = 2 * key_bytes;
    static constexpr size_t ts_off = acc_off + 2 * kN32 * sizeof(uint32_t);
    static constexpr size_t dbuf_off = ts_off + 2 * kN32 * sizeof(uint32_t);
    static constexpr size_t tw_off = dbuf_off + (size_t)GW * kN32 * sizeof(uint32_t);   // [fwd, inv][1024] uint2
    static constexpr size_t tables_off = tw_off + 2 * kN32 * sizeof(uint2);
    static size_t __host__ __device__ res_off(size_t tables) { return tables_off + (tables + 15) / 16 * 16; }
    static size_t __host__ __device__ bytes(size_t tables, size_t steps) { return res_off(tables) + (steps + 15) / 16 * 16; }
};

template <int DG>
__global__ void __launch_bounds__(32 * 2 * DG, 1)
    br32_solo_kernel(const __grid_constant__ PipeArgs A, const __grid_constant__ Ntt32Consts c,
                     const uint2 *__restrict__ fwd_tw, const uint2 *__restrict__ inv_tw, uint32_t mu32)
{
    using L = SoloLayout<DG>;
    constexpr int DT = DG - 1, GW = L::GW, NW = GW + 2, PT = 32 * NW;
    extern __shared__ __align__(16) unsigned char solo_smem[];
    __shared__ __align__(8) uint64_t bars[2];
    uint32_t(*acc)[kN32] = reinterpret_cast<uint32_t(*)[kN32]>(solo_smem + L::acc_off);
    uint32_t(*ts)[kN32] = reinterpret_cast<uint32_t(*)[kN32]>(solo_smem + L::ts_off);
    uint32_t(*dbuf)[kN32] = reinterpret_cast<uint32_t(*)[kN32]>(solo_smem + L::dbuf_off);
    uint2 *ftw = reinterpret_cast<uint2 *>(solo_smem + L::tw_off), *itw = ftw + kN32;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int S = A.n * (int)A.digitR;
    const int mode = issue_mode(A.flags);
    const size_t rgsw_words = (size_t)DG * 4 * kN32;

    for (int i = threadIdx.x; i < kN32; i += blockDim.x) {
        ftw[i] = __ldg(fwd_tw + i);
        itw[i] = __ldg(inv_tw + i);
    }
    const int cl = solo_table_copies_log2((int)A.bg_bits);
    const int BGC = A.digit_tables ? (1 << A.bg_bits) << cl : 0;
    uint32_t *t1 = reinterpret_cast<uint32_t *>(solo_smem + L::tables_off);
    uint2 *t23 = reinterpret_cast<uint2 *>(t1 + BGC), *t123 = t23 + BGC;
    uint8_t *res = solo_smem + L::res_off((size_t)(20 * BGC));
    for (int i = threadIdx.x; i < BGC; i += blockDim.x) {
        const uint64_t Q = c.Q, y = (uint64_t)(i >> cl);
        t1[i] = (uint32_t)(y * c.fw[1] % Q);
        t23[i] = make_uint2((uint32_t)(y * c.fw[2] % Q), (uint32_t)(y * c.fw[3] % Q));
        t123[i] = make_uint2((uint32_t)(y * A.w21 % Q), (uint32_t)(y * A.w31 % Q));
    }
    const DigitTables dt{t1, t23, t123, cl};
    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        mbar_fence_init();
    }
    __syncthreads();
    // bit b of parity: phase of bars[b] the next wait expects; of pending: a
    // copy into buffer b not yet waited for (thread 0, which issues the copies,
    // keeps the authoritative view)
    unsigned parity = 0, pending = 0;

    // the key of step s (residue res[s]) into buffer b
    auto fetch = [&](int s, int b) {
        pending |= 1u << b;
        const uint32_t *src = A.btkey + ((size_t)s * A.Br + res[s]) * rgsw_words;
        mbar_expect_tx(&bars[b], (unsigned)L::key_bytes);
#pragma unroll
        for (int h = 0; h < DG; h++)
            bulk_copy_g2s(solo_smem + b * L::key_bytes + h * (L::key_bytes / DG),
                          src + h * (rgsw_words / DG), (unsigned)(L::key_bytes / DG), &bars[b]);
    };

    for (size_t gid = blockIdx.x; gid < A.count; gid += gridDim.x) {
        // ---- LWE_evaluate, residues and the initial accumulator (global, B-tiled)
        if (warp == 0) pipe_init_item(A, c, fwd_tw, dbuf[0], res, gid, lane, mu32);
        __syncthreads();
        const int s0 = solo_next_step(res, -1, S, mode), s1 = s0 < S ? solo_next_step(res, s0, S, mode) : S;
        if (threadIdx.x == 0) {
            if (s0 < S) fetch(s0, 0);
            if (s1 < S) fetch(s1, 1);
        }
        {
            const uint4 *g4 = reinterpret_cast<const uint4 *>(A.accs + gid * 2048);
            for (int u = threadIdx.x; u < 512; u += PT) {
                const int P = u >> 8, v = u & 255;
                *reinterpret_cast<uint4 *>(acc[P] + sw_chunk(v & 31, v >> 5)) = __ldcg(g4 + u);
            }
        }
        __syncthreads();

        bool failed = false;
        int next = s1;   // the step whose key the buffer being released receives
        for (int s = s0, b = 0; s < S; b ^= 1) {
            if (warp >= GW) {
                const int hp = warp - GW;
                uint32_t x[32];
                load_row(x, acc[hp], lane);
                ntt_inv_1024_noscale<true>(x, c, itw, ts[hp], lane);
                store_row(ts[hp], lane, x);
            }
            __syncthreads();
            if (warp < GW) {
                const int p = warp / DT, h = warp % DT;
                const uint32_t shift = A.bg_bits * h, mask = (1u << A.bg_bits) - 1;
                uint32_t x[32];
                load_row(x, ts[p], lane);
#pragma unroll
                for (int r = 0; r < 32; r++) x[r] = (x[r] >> shift) & mask;
                if (A.digit_tables) ntt_fwd_1024_digit<true>(x, c, ftw, dbuf[warp], dt, lane);
                else ntt_fwd_1024<true>(x, c, ftw, dbuf[warp], lane);
                store_row(dbuf[warp], lane, x);
            }
            const bool ok = mbar_wait_bounded(&bars[b], (parity >> b) & 1u, kSoloWaitLimit);
            if (ok) {
                parity ^= 1u << b;
                pending &= ~(1u << b);
            }
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
            const uint4 *key = reinterpret_cast<const uint4 *>(solo_smem + b * L::key_bytes);
            for (int u = threadIdx.x; u < 256; u += PT) mac_chunk_solo<DG>(u, key, dbuf, acc, c.Q, A.qinv_neg);
            __syncthreads();
            // buffer b is free again: it receives the key after the one in flight
            const int after = next < S ? solo_next_step(res, next, S, mode) : S;
            if (threadIdx.x == 0 && after < S) fetch(after, b);
            s = next;
            next = after;
        }
        if (failed) {
            // flag the launch, let the copies in flight land (the CTA's shared
            // memory stays allocated while thread 0 waits), and stop
            if (threadIdx.x == 0) {
                atomicOr(A.status, kStatusWaitLimit);
                for (int b = 0; b < 2; b++)
                    if (pending & (1u << b)) mbar_wait_bounded(&bars[b], (parity >> b) & 1u, kSoloWaitLimit);
            }
            return;
        }

        // ---- accumulator back to global memory, then the outputs of the pipelines' epilogue
        {
            uint4 *g4 = reinterpret_cast<uint4 *>(A.accs + gid * 2048);
            for (int u = threadIdx.x; u < 512; u += PT) {
                const int P = u >> 8, v = u & 255;
                __stcg(g4 + u, *reinterpret_cast<const uint4 *>(acc[P] + sw_chunk(v & 31, v >> 5)));
            }
        }
        __syncthreads();
        if (warp < 2) pipe_out_poly(A, c, inv_tw, dbuf[warp], gid, warp, lane);
        __syncthreads();
    }
}

}  // namespace dev

static int sm_count(Context &c)
{
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, c.device);
    return v > 0 ? v : 1;
}

template <int DG, int NP, int MINB>
static int launch_pipe_dg(Context &c, dev::PipeArgs A, int max_ctas, cudaStream_t st)
{
    constexpr int GW = 2 * (DG - 1);
    constexpr int threads = NP * 32 * (GW + 2);
    auto kern = dev::br32_pipe_kernel<DG, NP, MINB>;
    const size_t steps = (size_t)c.p.n * c.p.digitR;
    const size_t tables = A.digit_tables ? (20 * ((size_t)1 << c.p.BG_bits)) << dev::digit_table_copies_log2((int)c.p.BG_bits) : 0;
    // group cap: kMaxGroup (or the tuned cap) per pipeline, within the shared memory of one CTA
    int cap = NP * (c.tune.br_group > 0 ? std::min(c.tune.br_group, dev::kMaxGroup) : dev::kMaxGroup);
    const size_t fixed = dev::pipe_tables_offset<GW, NP>(0, steps) + tables + 16;
    if (fixed + (size_t)cap * steps > kPipeSmemBudget)
        cap = fixed < kPipeSmemBudget ? (int)((kPipeSmemBudget - fixed) / steps) : 0;
    if (cap < 1) return c.fail(FHEACC_EINVAL, "n * digitR too large for the blind rotation's residue table");
    // residency with the largest group allowed; the group is then fitted to the batch
    size_t smem = dev::pipe_tables_offset<GW, NP>(cap, steps) + tables;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return c.cuda_fail(e, "blind rotation smem attribute");
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
    if (per_sm < 1) per_sm = 1;
    if (c.tune.br_ctas_per_sm > 0) per_sm = std::min(per_sm, c.tune.br_ctas_per_sm);
    // at least two ciphertexts per pipeline keep both of its stages busy
    size_t blocks = std::min<size_t>((size_t)sm_count(c) * per_sm, (A.count + 2 * NP - 1) / (2 * NP));
    if (max_ctas > 0) blocks = std::min<size_t>(blocks, (size_t)max_ctas);
    blocks = std::max<size_t>(blocks, 1);
    // equal claims: the fewest rounds of at most `cap` ciphertexts per CTA
    const size_t rounds = (A.count + blocks * cap - 1) / (blocks * cap);
    A.group = (int)((A.count + blocks * rounds - 1) / (blocks * rounds));
    smem = dev::pipe_tables_offset<GW, NP>(A.group, steps) + tables;
    // claim counter after the accumulators
    A.claim_next = reinterpret_cast<unsigned long long *>(A.accs + A.count * 2048);
    e = cudaMemsetAsync(A.claim_next, 0, kClaimWords * sizeof(uint32_t), st);
    if (e != cudaSuccess) return c.cuda_fail(e, "blind rotation claim reset");
    kern<<<(unsigned)blocks, threads, smem, st>>>(A, c.nc, c.d_fwd_tw, c.d_inv_tw, (uint32_t)((1ULL << 32) / c.p.Q));
    c.launches++;
    e = cudaGetLastError();
    return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "blind rotation launch");
}

// Latency form: one CTA per ciphertext on up to one CTA per SM, each CTA
// taking every gridDim-th ciphertext.
template <int DG>
static int launch_solo_dg(Context &c, const dev::PipeArgs &A, int max_ctas, cudaStream_t st)
{
    using L = dev::SoloLayout<DG>;
    constexpr int threads = 32 * 2 * DG;
    auto kern = dev::br32_solo_kernel<DG>;
    const size_t steps = (size_t)c.p.n * c.p.digitR;
    const size_t tables = A.digit_tables ? (20 * ((size_t)1 << c.p.BG_bits)) << dev::solo_table_copies_log2((int)c.p.BG_bits) : 0;
    const size_t smem = L::bytes(tables, steps);
    if (smem > kPipeSmemBudget) return 1;   // does not fit: the caller takes the pipelines
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return c.cuda_fail(e, "blind rotation (latency form) smem attribute");
    size_t blocks = std::min<size_t>(A.count, (size_t)sm_count(c));
    if (max_ctas > 0) blocks = std::min<size_t>(blocks, (size_t)max_ctas);
    kern<<<(unsigned)blocks, threads, smem, st>>>(A, c.nc, c.d_fwd_tw, c.d_inv_tw, (uint32_t)((1ULL << 32) / c.p.Q));
    c.launches++;
    e = cudaGetLastError();
    return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "blind rotation (latency form) launch");
}

// Latency form up to this many gates per SM by default (one GB300, 4096-gate
// key set); FHEACC_OPT_BR_SOLO overrides, 0 turns it off.
constexpr int kSoloGatesPerSm = 1;

// Pipelines per CTA. By default from the gates per SM (one GB300, 4096-gate
// key set): up to 2 a single pipeline per SM is fastest (its items do not
// wait on other pipelines), up to 5 two pipelines, beyond that three.
template <int DG>
static int launch_pipe_shape(Context &c, const dev::PipeArgs &A, int max_ctas, cudaStream_t st)
{
    const size_t sms = (size_t)sm_count(c);
    // explicit pipeline shapes and the wait-limit tests keep the pipelines
    const int solo = c.tune.br_solo >= 0 ? c.tune.br_solo : kSoloGatesPerSm;
    if (solo > 0 && c.tune.br_pipes == 0 && c.tune.debug_wait_limit < 0 && A.count <= (size_t)solo * sms) {
        const int rc = launch_solo_dg<DG>(c, A, max_ctas, st);
        if (rc != 1) return rc;
    }
    const int np = c.tune.br_pipes > 0 ? c.tune.br_pipes : A.count <= 2 * sms ? 1 : A.count <= 5 * sms ? 2 : 3;
    if (np == 3) return launch_pipe_dg<DG, 3, 1>(c, A, max_ctas, st);
    if (np == 2) return launch_pipe_dg<DG, 2, 1>(c, A, max_ctas, st);
    // one pipeline per CTA: the register budget of 3 (default) or 2 CTAs per SM
    return c.tune.br_regs_for_3 != 0 ? launch_pipe_dg<DG, 1, 3>(c, A, max_ctas, st)
                                     : launch_pipe_dg<DG, 1, 2>(c, A, max_ctas, st);
}

// Parameter-set fields of PipeArgs.
static void fill_pipe_params(Context &c, dev::PipeArgs &A, uint32_t flags)
{
    const uint64_t Q = c.p.Q;
    A.btkey = c.d_btkey;
    A.n = c.p.n; A.q = c.p.q; A.embed = c.dp.embed; A.Br = c.p.Br; A.digitR = c.p.digitR;
    A.bg_bits = c.p.BG_bits; A.flags = flags;
    A.qinv_neg = c.dp.qinv_neg;
    A.tv_pos = (uint32_t)((unsigned __int128)(Q / 8 + 1) * c.p.iN % Q);
    A.tv_neg = (uint32_t)(Q - A.tv_pos);
    A.nmul = (uint32_t)(c.p.N % Q);
    A.nmuls = (uint32_t)(((uint64_t)A.nmul << 32) / Q);
    A.w21 = (uint32_t)((uint64_t)c.nc.fw[2] * c.nc.fw[1] % Q);
    A.w31 = (uint32_t)((uint64_t)c.nc.fw[3] * c.nc.fw[1] % Q);
    A.derive_last = c.dp.last_digit_from_acc;
    A.status = c.d_status;
    A.idle_limit = c.tune.debug_wait_limit >= 0 ? c.tune.debug_wait_limit : dev::kIdleLimit;
    A.digit_tables = (1u << c.p.BG_bits) <= (uint32_t)dev::kMaxTableBG;
    for (int i = 0; i < 8; i++) A.gate_constant[i] = c.dp.gate_constant[i];
}

static int launch_pipe(Context &c, const dev::PipeArgs &A, int max_ctas, cudaStream_t st)
{
    // parameter validation makes the gadget cover Q, which the last-digit
    // identity of the kernel needs
    if (!A.derive_last) return c.fail(FHEACC_EINVAL, "gadget base^digitG must exceed Q");
    switch (c.p.digitG) {
    case 2: return launch_pipe_shape<2>(c, A, max_ctas, st);
    case 3: return launch_pipe_shape<3>(c, A, max_ctas, st);
    case 4: return launch_pipe_shape<4>(c, A, max_ctas, st);
    default: return c.fail(FHEACC_EINVAL, "digitG must be 2..4 for the 32-bit path");
    }
}

int launch_blind_rotate32(Context &c, const uint64_t *d_c1, const uint64_t *d_c2, const int32_t *d_gates,
                          size_t count, uint32_t flags, uint64_t *d_acc_out, uint32_t *d_extract, int max_ctas,
                          cudaStream_t st)
{
    if (!count) return FHEACC_OK;
    if (!c.d_btkey) return c.fail(FHEACC_ENOKEY, "bootstrap key not uploaded");
    int rc = ensure_scratch(c, c.accs, bootstrap_accs_bytes(c, count));
    if (rc) return rc;
    dev::PipeArgs A{};
    A.c1 = d_c1; A.c2 = d_c2; A.gates = d_gates; A.count = count;
    A.accs = (uint32_t *)c.accs.ptr; A.acc_out = d_acc_out; A.extract = d_extract;
    fill_pipe_params(c, A, flags);
    return launch_pipe(c, A, max_ctas, st);
}

}  // namespace fheacc

namespace fheacc {

// Same launch as launch_blind_rotate32, with the accumulator scratch supplied
// by the caller (`accs`: bootstrap_accs_bytes, 16-byte aligned); allocates
// nothing.
int launch_blind_rotate32_with(Context &c, const uint64_t *d_c1, const uint64_t *d_c2, const int32_t *d_gates,
                               size_t count, uint32_t flags, uint32_t *accs, uint32_t *d_extract, cudaStream_t st)
{
    return launch_blind_rotate32_indexed(c, d_c1, d_c2, nullptr, nullptr, d_gates, count, flags, accs, d_extract, st);
}

int launch_blind_rotate32_indexed(Context &c, const uint64_t *d_c1, const uint64_t *d_c2, const uint32_t *d_idx1,
                                  const uint32_t *d_idx2, const int32_t *d_gates, size_t count, uint32_t flags,
                                  uint32_t *accs, uint32_t *d_extract, cudaStream_t st)
{
    if (!count) return FHEACC_OK;
    if (!c.d_btkey) return c.fail(FHEACC_ENOKEY, "bootstrap key not uploaded");
    dev::PipeArgs A{};
    A.c1 = d_c1; A.c2 = d_c2; A.idx1 = d_idx1; A.idx2 = d_idx2; A.gates = d_gates; A.count = count;
    A.accs = accs; A.acc_out = nullptr; A.extract = d_extract;
    fill_pipe_params(c, A, flags);
    return launch_pipe(c, A, 0, st);
}

}  // namespace fheacc
