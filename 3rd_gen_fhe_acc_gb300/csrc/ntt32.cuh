// ntt32.cuh -- one-warp negacyclic NTT / inverse NTT of a 1024-point
// polynomial with 32-bit words, for Q < 2^27.
//
// Computes exactly the transforms of the reference's NTT / iNTT
// (FHE_ACC_runtime/src/nbt.cpp:423-454 and 456-491: Cooley-Tukey with the
// bit-reversed psi table, Gentleman-Sande with the bit-reversed psi^-1 table
// and a final *N^-1), so canonical outputs are bit-identical.
//
// Data layout: each lane holds 32 coefficients in registers.
//   layout A: lane l, register r holds element  l + 32 r   (strided)
//   layout B: lane l, register r holds element 32 l + r    (contiguous)
// The forward transform runs its first five stages (t = 512..32) in layout A,
// where every lane uses the same twiddle (taken from the kernel's parameter
// bank), one padded shared-memory transpose, and the last five stages
// (t = 16..1) in layout B with per-lane twiddles read through L1 from
// lane-interleaved tables (coalesced warp loads). The inverse
// runs the same way backwards. The transpose goes through a swizzled shared-
// memory tile: rows move as 128-bit chunks, columns as conflict-free words.
//
// Modular arithmetic: Shoup multiplication by precomputed (w, w' =
// floor(w 2^32 / Q)) gives x*w mod Q in [0, 2Q) for any 32-bit x. The forward
// butterflies never reduce the upper input: each stage adds at most 2Q to the
// bound, so inputs below Q leave the transform below 21Q < 2^32 (Q < 2^27).
// The inverse keeps Harvey's [0, 2Q) invariant and ends canonical.
#pragma once
#include <cstdint>

namespace fheacc {
namespace dev {

constexpr int kN32 = 1024;
constexpr int kPadN = 1024 + 32;   // padded words per polynomial in shared memory

// Warp-uniform twiddles (stages with m < 32), passed in the kernel's parameter
// bank so that fully unrolled stages read them as constant operands.
struct Ntt32Consts {
    uint32_t Q, twoQ;
    uint32_t fw[32], fws[32];    // rou[m+i],  m+i < 32, and Shoup companions
    uint32_t iw[32], iws[32];    // irou[m+i], m+i < 32
    uint32_t iN, iNs;            // N^-1
    uint32_t iw1N, iw1Ns;        // irou[1] * N^-1
};

__device__ __forceinline__ int pad32(int e) { return e + (e >> 5); }

__device__ __forceinline__ uint32_t shoup32(uint32_t x, uint32_t w, uint32_t ws, uint32_t Q)
{
    uint32_t t = __umulhi(x, ws);
    return x * w - t * Q;   // in [0, 2Q)
}

// Cooley-Tukey butterfly, upper input left unreduced.
__device__ __forceinline__ void ct_bfly(uint32_t &x, uint32_t &y, uint32_t w, uint32_t ws, uint32_t Q,
                                        uint32_t twoQ)
{
    uint32_t t = shoup32(y, w, ws, Q);
    y = x + twoQ - t;
    x = x + t;
}

// Gentleman-Sande butterfly, inputs and outputs in [0, 2Q).
__device__ __forceinline__ void gs_bfly(uint32_t &x, uint32_t &y, uint32_t w, uint32_t ws, uint32_t Q,
                                        uint32_t twoQ)
{
    uint32_t u = x + y;
    u = min(u, u - twoQ);
    uint32_t v = shoup32(x - y + twoQ, w, ws, Q);
    x = u;
    y = v;
}

// Forward stage s (0..4) in layout A.
template <int S>
__device__ __forceinline__ void fwd_stage_A(uint32_t (&x)[32], const Ntt32Consts &c)
{
    constexpr int h = 16 >> S, m = 1 << S;
#pragma unroll
    for (int r = 0; r < 32; r++) {
        if (!(r & h)) {
            const int i = r / (2 * h);
            ct_bfly(x[r], x[r + h], c.fw[m + i], c.fws[m + i], c.Q, c.twoQ);
        }
    }
}

// Per-lane twiddles of the layout-B stages come from "lane-interleaved"
// tables (built by the host, see fheacc::build_tables): a stage in which every
// lane needs G consecutive table entries m + G*lane + g stores entry (g, lane)
// at (g / 2) * 64 + 2 * lane + g % 2, so each warp load reads 256 or 512
// contiguous bytes. Forward stages s = 5..9 (G = 1..16) start at
// 32 * (2^(s-5) - 1); inverse stages t = 1..16 (G = 16/t) at 32 * (32 - 32/t).
// Both tables have 992 entries. SH: the table is a copy in shared memory
// (plain loads) instead of global memory read through L1 (__ldg).
template <int G, int OFF, bool SH = false>
__device__ __forceinline__ void load_stage_twiddles(uint2 (&w)[G], const uint2 *__restrict__ tw, int lane)
{
    if (G == 1) {
        w[0] = SH ? tw[OFF + lane] : __ldg(tw + OFF + lane);
    } else {
        const uint4 *t4 = reinterpret_cast<const uint4 *>(tw + OFF);
#pragma unroll
        for (int gg = 0; gg < G / 2; gg++) {
            const uint4 v = SH ? t4[gg * 32 + lane] : __ldg(t4 + gg * 32 + lane);
            w[2 * gg] = make_uint2(v.x, v.y);
            w[2 * gg + 1] = make_uint2(v.z, v.w);
        }
    }
}

// Forward stage s (5..9) in layout B.
template <int S, bool SH = false>
__device__ __forceinline__ void fwd_stage_B(uint32_t (&x)[32], const uint2 *__restrict__ tw, int lane,
                                            uint32_t Q, uint32_t twoQ)
{
    constexpr int t = 512 >> S, G = 16 / t;   // G twiddles per lane
    uint2 w[G];
    load_stage_twiddles<G, 32 * ((1 << (S - 5)) - 1), SH>(w, tw, lane);
#pragma unroll
    for (int r = 0; r < 32; r++) {
        if (!(r & t)) {
            const int g = r / (2 * t);
            ct_bfly(x[r], x[r + t], w[g].x, w[g].y, Q, twoQ);
        }
    }
}

// Inverse stage with butterfly distance t (1..16) in layout B.
template <int T, bool SH = false>
__device__ __forceinline__ void inv_stage_B(uint32_t (&x)[32], const uint2 *__restrict__ tw, int lane,
                                            uint32_t Q, uint32_t twoQ)
{
    constexpr int G = 16 / T;
    uint2 w[G];
    load_stage_twiddles<G, 32 * (32 - 32 / T), SH>(w, tw, lane);
#pragma unroll
    for (int r = 0; r < 32; r++) {
        if (!(r & T)) {
            const int g = r / (2 * T);
            gs_bfly(x[r], x[r + T], w[g].x, w[g].y, Q, twoQ);
        }
    }
}

// Inverse stage with butterfly distance t = 32*H (H = 1..8) in layout A.
template <int H>
__device__ __forceinline__ void inv_stage_A(uint32_t (&x)[32], const Ntt32Consts &c)
{
    constexpr int m = 16 / H;
#pragma unroll
    for (int r = 0; r < 32; r++) {
        if (!(r & H)) {
            const int i = r / (2 * H);
            gs_bfly(x[r], x[r + H], c.iw[m + i], c.iws[m + i], c.Q, c.twoQ);
        }
    }
}

// Swizzled 32 x 32 tile of a 1024-word poly (no padding): element e in row
// e / 32, column e % 32 sits at  row * 32 + ((col / 4) ^ (row % 8)) * 4 + col % 4.
// A lane reading or writing a whole row (layout B, or any lane-major copy)
// moves 8 conflict-free 128-bit chunks; a warp touching one element of every
// column of a row (layout A) hits 32 distinct banks.
__device__ __forceinline__ int sw_addr(int row, int col) { return (row << 5) + ((((col >> 2) ^ (row & 7))) << 2) + (col & 3); }
__device__ __forceinline__ int sw_chunk(int row, int k) { return (row << 5) + ((k ^ (row & 7)) << 2); }

__device__ __forceinline__ void store_row(uint32_t *buf, int row, const uint32_t (&x)[32])
{
#pragma unroll
    for (int k = 0; k < 8; k++)
        *reinterpret_cast<uint4 *>(buf + sw_chunk(row, k)) = make_uint4(x[4 * k], x[4 * k + 1], x[4 * k + 2], x[4 * k + 3]);
}

__device__ __forceinline__ void load_row(uint32_t (&x)[32], const uint32_t *buf, int row)
{
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const uint4 v = *reinterpret_cast<const uint4 *>(buf + sw_chunk(row, k));
        x[4 * k] = v.x; x[4 * k + 1] = v.y; x[4 * k + 2] = v.z; x[4 * k + 3] = v.w;
    }
}

// Layout A -> B through a per-warp buffer of 1024 words (16-byte aligned).
__device__ __forceinline__ void transpose_A_to_B(uint32_t (&x)[32], uint32_t *buf, int lane)
{
    __syncwarp();
#pragma unroll
    for (int r = 0; r < 32; r++) buf[sw_addr(r, lane)] = x[r];
    __syncwarp();
    load_row(x, buf, lane);
    __syncwarp();
}

__device__ __forceinline__ void transpose_B_to_A(uint32_t (&x)[32], uint32_t *buf, int lane)
{
    __syncwarp();
    store_row(buf, lane, x);
    __syncwarp();
#pragma unroll
    for (int r = 0; r < 32; r++) x[r] = buf[sw_addr(r, lane)];
    __syncwarp();
}

// Forward NTT: x in layout A (values < Q) -> layout B, values < 21Q, in the
// reference's bit-reversed output order. buf: 1024 words of 16-byte aligned
// scratch. SH: fwd_tw is a shared-memory copy of the table.
template <bool SH = false>
__device__ __forceinline__ void ntt_fwd_1024(uint32_t (&x)[32], const Ntt32Consts &c,
                                             const uint2 *__restrict__ fwd_tw, uint32_t *buf, int lane)
{
    fwd_stage_A<0>(x, c);
    fwd_stage_A<1>(x, c);
    fwd_stage_A<2>(x, c);
    fwd_stage_A<3>(x, c);
    fwd_stage_A<4>(x, c);
    transpose_A_to_B(x, buf, lane);
    fwd_stage_B<5, SH>(x, fwd_tw, lane, c.Q, c.twoQ);
    fwd_stage_B<6, SH>(x, fwd_tw, lane, c.Q, c.twoQ);
    fwd_stage_B<7, SH>(x, fwd_tw, lane, c.Q, c.twoQ);
    fwd_stage_B<8, SH>(x, fwd_tw, lane, c.Q, c.twoQ);
    fwd_stage_B<9, SH>(x, fwd_tw, lane, c.Q, c.twoQ);
}

// Products of a gadget digit (y < BG) with the three twiddles of the first two
// forward stages, which are the same for every lane: w1 = rou[1] (stage t =
// 512), w2 = rou[2] and w3 = rou[3] (stage t = 256). The tables hold, for
// y < BG:  t1[y] = y w1,  t23[y] = (y w2, y w3),  t123[y] = (y w2 w1, y w3 w1),
// all canonical mod Q. Each table is held in 2^copies_log2 copies, entry y of
// copy k at [(y << copies_log2) + k], and lane l reads copy l mod 2^copies_log2:
// with 16 copies the digits of a warp (random 7-bit values) hit distinct banks
// in the 64-bit tables and at most two lanes share a bank in t1, instead of
// several lanes per bank for a single copy.
struct DigitTables {
    const uint32_t *t1;
    const uint2 *t23, *t123;
    int copies_log2;
};

// Copies of the digit tables a gadget base of 2^bg_bits gets (shared memory
// 20 BG bytes per copy: 16 copies up to BG = 128).
__host__ __device__ constexpr int digit_table_copies_log2(int bg_bits) { return bg_bits <= 7 ? 4 : 0; }

// Forward NTT of a digit polynomial: x in layout A with values < BG -> layout
// B, values < 19Q + BG, same result mod Q as ntt_fwd_1024. The first two
// stages form, for r < 8, the radix-4 group (x0, x1, x2, x3) = x[r, r+8, r+16,
// r+24]:
//   x[r]      = x0 + w1 x2 + w2 x1 + w2 w1 x3
//   x[r + 8]  = x0 + w1 x2 - w2 x1 - w2 w1 x3
//   x[r + 16] = x0 - w1 x2 + w3 x1 - w3 w1 x3
//   x[r + 24] = x0 - w1 x2 - w3 x1 + w3 w1 x3
// with the five products read from DigitTables (three shared-memory loads
// instead of four Shoup multiplies), each output below 3Q + BG.
template <bool SH = false>
__device__ __forceinline__ void ntt_fwd_1024_digit(uint32_t (&x)[32], const Ntt32Consts &c,
                                                   const uint2 *__restrict__ fwd_tw, uint32_t *buf,
                                                   const DigitTables &T, int lane)
{
    const int cl = T.copies_log2, cp = lane & ((1 << cl) - 1);
#pragma unroll
    for (int r = 0; r < 8; r++) {
        const uint32_t x0 = x[r], x1 = x[r + 8], x2 = x[r + 16], x3 = x[r + 24];
        const uint32_t a = T.t1[(x2 << cl) + cp];
        const uint2 bd = T.t23[(x1 << cl) + cp], ce = T.t123[(x3 << cl) + cp];
        x[r] = x0 + a + bd.x + ce.x;
        x[r + 8] = x0 + a + (c.twoQ - bd.x - ce.x);
        x[r + 16] = x0 + (c.twoQ - a - ce.y) + bd.y;
        x[r + 24] = x0 + (c.twoQ - a - bd.y) + ce.y;
    }
    fwd_stage_A<2>(x, c);
    fwd_stage_A<3>(x, c);
    fwd_stage_A<4>(x, c);
    transpose_A_to_B(x, buf, lane);
    fwd_stage_B<5, SH>(x, fwd_tw, lane, c.Q, c.twoQ);
    fwd_stage_B<6, SH>(x, fwd_tw, lane, c.Q, c.twoQ);
    fwd_stage_B<7, SH>(x, fwd_tw, lane, c.Q, c.twoQ);
    fwd_stage_B<8, SH>(x, fwd_tw, lane, c.Q, c.twoQ);
    fwd_stage_B<9, SH>(x, fwd_tw, lane, c.Q, c.twoQ);
}

// Inverse NTT without the final N^-1: x in layout B (values < 2Q) -> layout
// A, canonical, equal to N * (the reference's iNTT) mod Q. Used on
// accumulators that already carry the factor N^-1 (bootstrap keys uploaded
// times N^-1). SH: inv_tw is a shared-memory copy of the table.
template <bool SH = false>
__device__ __forceinline__ void ntt_inv_1024_noscale(uint32_t (&x)[32], const Ntt32Consts &c,
                                                     const uint2 *__restrict__ inv_tw, uint32_t *buf, int lane)
{
    inv_stage_B<1, SH>(x, inv_tw, lane, c.Q, c.twoQ);
    inv_stage_B<2, SH>(x, inv_tw, lane, c.Q, c.twoQ);
    inv_stage_B<4, SH>(x, inv_tw, lane, c.Q, c.twoQ);
    inv_stage_B<8, SH>(x, inv_tw, lane, c.Q, c.twoQ);
    inv_stage_B<16, SH>(x, inv_tw, lane, c.Q, c.twoQ);
    transpose_B_to_A(x, buf, lane);
    inv_stage_A<1>(x, c);
    inv_stage_A<2>(x, c);
    inv_stage_A<4>(x, c);
    inv_stage_A<8>(x, c);
#pragma unroll
    for (int r = 0; r < 16; r++) {
        uint32_t u = x[r] + x[r + 16];
        u = min(u, u - c.twoQ);
        const uint32_t v = shoup32(x[r] - x[r + 16] + c.twoQ, c.iw[1], c.iws[1], c.Q);
        x[r] = min(u, u - c.Q);
        x[r + 16] = min(v, v - c.Q);
    }
}

// Inverse NTT: x in layout B (values < 2Q, bit-reversed order) -> layout A,
// canonical time-domain coefficients (times N^-1).
__device__ __forceinline__ void ntt_inv_1024(uint32_t (&x)[32], const Ntt32Consts &c,
                                             const uint2 *__restrict__ inv_tw, uint32_t *buf, int lane)
{
    inv_stage_B<1>(x, inv_tw, lane, c.Q, c.twoQ);
    inv_stage_B<2>(x, inv_tw, lane, c.Q, c.twoQ);
    inv_stage_B<4>(x, inv_tw, lane, c.Q, c.twoQ);
    inv_stage_B<8>(x, inv_tw, lane, c.Q, c.twoQ);
    inv_stage_B<16>(x, inv_tw, lane, c.Q, c.twoQ);
    transpose_B_to_A(x, buf, lane);
    inv_stage_A<1>(x, c);
    inv_stage_A<2>(x, c);
    inv_stage_A<4>(x, c);
    inv_stage_A<8>(x, c);
    // last stage (t = 512, m = 1) with N^-1 folded into both outputs
#pragma unroll
    for (int r = 0; r < 16; r++) {
        uint32_t u = shoup32(x[r] + x[r + 16], c.iN, c.iNs, c.Q);
        uint32_t v = shoup32(x[r] - x[r + 16] + c.twoQ, c.iw1N, c.iw1Ns, c.Q);
        x[r] = min(u, u - c.Q);
        x[r + 16] = min(v, v - c.Q);
    }
}

}  // namespace dev
}  // namespace fheacc
