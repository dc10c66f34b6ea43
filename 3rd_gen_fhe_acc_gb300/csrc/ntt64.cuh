// ntt64.cuh -- negacyclic NTT / inverse NTT of a 2048-point polynomial with
// 64-bit words (Q < 2^62), computed in shared memory by a group of threads.
//
// Same transforms as the reference's NTT / iNTT (FHE_ACC_runtime/src/
// nbt.cpp:423-454 and 456-491), so canonical outputs are bit-identical.
//
// A 64-bit Shoup multiplication (w' = floor(w 2^64 / Q)) costs about five
// times a 32-bit one, so shared-memory traffic matters less here than in the
// 32-bit path: the polynomial stays in shared memory and each thread runs
// radix-8 / radix-16 passes (three or four butterfly stages per load/store of
// 8 or 16 words: 3 passes per forward transform, 4 per inverse), with one
// group barrier per pass.
// Forward butterflies leave the upper input unreduced
// (bound grows by 2Q a stage: inputs < Q end below 23Q < 2^59 for Q < 2^54);
// the inverse keeps Harvey's [0, 2Q) invariant and ends canonical.
#pragma once
#include <cstdint>

namespace fheacc {
namespace dev {

// Shared-memory layouts of a 2048-word polynomial, chosen by the template
// parameter P of the transforms: P = false, word e at e; P = true, one padding
// word after every 8, word e at px(e). Padded, the passes whose threads walk 8
// consecutive words (the last forward and the first inverse pass) spread a
// warp over all banks instead of two bank pairs; the offsets of a pass's tuple
// stay linear in the tuple index (strides 1 within an octet, or multiples of
// 8). The padding costs shared memory, hence L1, which only some kernels spare.
constexpr int kPoly64 = 2048 + 256;
__host__ __device__ __forceinline__ int px(int e) { return e + (e >> 3); }
template <bool P>
__host__ __device__ __forceinline__ int pi(int e) { return P ? px(e) : e; }
template <bool P>
__host__ __device__ constexpr int poly_words64() { return P ? kPoly64 : 2048; }

struct Ntt64Consts {
    uint64_t Q, twoQ;
    uint64_t iN, iNs;       // N^-1 and its Shoup companion
    uint64_t iw1N, iw1Ns;   // irou[1] * N^-1
    uint64_t mu64;          // floor(2^64 / Q)
};

__device__ __forceinline__ uint64_t shoup64(uint64_t x, uint64_t w, uint64_t ws, uint64_t Q)
{
    const uint64_t t = __umul64hi(x, ws);
    return x * w - t * Q;   // in [0, 2Q)
}

__device__ __forceinline__ void ct64(uint64_t &x, uint64_t &y, ulonglong2 w, uint64_t Q, uint64_t twoQ)
{
    const uint64_t t = shoup64(y, w.x, w.y, Q);
    y = x + twoQ - t;
    x = x + t;
}

__device__ __forceinline__ void gs64(uint64_t &x, uint64_t &y, ulonglong2 w, uint64_t Q, uint64_t twoQ)
{
    uint64_t u = x + y;
    u = u >= twoQ ? u - twoQ : u;
    const uint64_t v = shoup64(x - y + twoQ, w.x, w.y, Q);
    x = u;
    y = v;
}

// x < 2^64 -> [0, 2Q)
__device__ __forceinline__ uint64_t barrett64_2q(uint64_t x, uint64_t mu64, uint64_t Q)
{
    return x - __umul64hi(x, mu64) * Q;
}

__device__ __forceinline__ void group_sync(int bar_id, int threads)
{
    asm volatile("bar.sync %0, %1;" ::"r"(bar_id), "r"(threads) : "memory");
}

// One radix-2^R forward pass: stages t, t/2, ..., t/2^(R-1) (m = N / 2t) on
// the tuples e0 + k t/2^(R-1) (k < 2^R) of every 2t-block.
template <int G, int R, bool P>
__device__ __forceinline__ void fwd_passR(uint64_t *a, const ulonglong2 *__restrict__ tw, const Ntt64Consts &c,
                                          int tid, int t, int m)
{
    constexpr int K = 1 << R;
    const int h = t >> (R - 1);
    for (int oc = tid; oc < 2048 / K; oc += G) {
        const int grp = oc / h, j = oc - grp * h;
        const int e0 = grp * 2 * t + j;
        uint64_t x[K];
#pragma unroll
        for (int k = 0; k < K; k++) x[k] = a[pi<P>(e0 + k * h)];
#pragma unroll
        for (int st = 0; st < R; st++) {
            const int d = K >> (st + 1);
#pragma unroll
            for (int k = 0; k < K; k++) {
                if (k & d) continue;
                ct64(x[k], x[k + d], __ldg(tw + (m << st) + (grp << st) + (k >> (R - st))), c.Q, c.twoQ);
            }
        }
#pragma unroll
        for (int k = 0; k < K; k++) a[pi<P>(e0 + k * h)] = x[k];
    }
}

// Forward NTT of a[poly_words64<P>()] (layout pi<P>) in shared memory by `G` threads (tid < G) that share
// the named barrier `bar`. tw[k] = (psi^bitrev(k), companion). Input < Q,
// output < 23Q, bit-reversed order as the reference's. Two radix-16 passes
// (stages t = 1024..128, 64..8) and one radix-8 pass (t = 4, 2, 1).
template <int G, bool P>
__device__ __forceinline__ void ntt64_fwd_2048(uint64_t *a, const ulonglong2 *__restrict__ tw, const Ntt64Consts &c,
                                               int tid, int bar)
{
    fwd_passR<G, 4, P>(a, tw, c, tid, 1024, 1);   // t = 1024 .. 128
    group_sync(bar, G);
    fwd_passR<G, 4, P>(a, tw, c, tid, 64, 16);    // t = 64 .. 8
    group_sync(bar, G);
    fwd_passR<G, 3, P>(a, tw, c, tid, 4, 256);    // t = 4, 2, 1
    group_sync(bar, G);
}

// Products of a gadget digit (y < BG) with the three twiddles of the first two
// forward stages, w1 = psi^bitrev(1) (stage t = 1024), w2 and w3 (t = 512):
// t1[y] = y w1, t23[y] = (y w2, y w3), t123[y] = (y w2 w1, y w3 w1), mod Q.
struct DigitTables64 {
    const uint64_t *t1;
    const ulonglong2 *t23, *t123;
};

// First forward pass (stages t = 1024 .. 128) of a digit polynomial (values
// < BG): the first two stages of each radix-4 group (x0, x1, x2, x3) =
// x[r, r+4, r+8, r+12] of a 16-tuple come from the tables,
//   x[r]      = x0 + w1 x2 + w2 x1 + w2 w1 x3
//   x[r + 4]  = x0 + w1 x2 - w2 x1 - w2 w1 x3
//   x[r + 8]  = x0 - w1 x2 + w3 x1 - w3 w1 x3
//   x[r + 12] = x0 - w1 x2 - w3 x1 + w3 w1 x3
// (each below 3Q + BG), the other two stages are Cooley-Tukey butterflies.
template <int G, bool P>
__device__ __forceinline__ void fwd_pass16_digit(uint64_t *a, const ulonglong2 *__restrict__ tw, const Ntt64Consts &c,
                                                 int tid, const DigitTables64 &T)
{
    for (int j = tid; j < 128; j += G) {
        uint64_t x[16];
#pragma unroll
        for (int k = 0; k < 16; k++) x[k] = a[pi<P>(j + k * 128)];
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const uint64_t x0 = x[r];
            const uint64_t av = T.t1[x[r + 8]];
            const ulonglong2 bd = T.t23[x[r + 4]], ce = T.t123[x[r + 12]];
            x[r] = x0 + av + bd.x + ce.x;
            x[r + 4] = x0 + av + (c.twoQ - bd.x - ce.x);
            x[r + 8] = x0 + (c.twoQ - av - ce.y) + bd.y;
            x[r + 12] = x0 + (c.twoQ - av - bd.y) + ce.y;
        }
#pragma unroll
        for (int st = 2; st < 4; st++) {
            const int d = 16 >> (st + 1);
#pragma unroll
            for (int k = 0; k < 16; k++) {
                if (k & d) continue;
                ct64(x[k], x[k + d], __ldg(tw + (1 << st) + (k >> (4 - st))), c.Q, c.twoQ);
            }
        }
#pragma unroll
        for (int k = 0; k < 16; k++) a[pi<P>(j + k * 128)] = x[k];
    }
}

// Forward NTT of a digit polynomial (values < BG) as ntt64_fwd_2048, the
// first two stages from the digit tables; output < 21Q + BG.
template <int G, bool P>
__device__ __forceinline__ void ntt64_fwd_2048_digit(uint64_t *a, const ulonglong2 *__restrict__ tw,
                                                     const Ntt64Consts &c, int tid, int bar, const DigitTables64 &T)
{
    fwd_pass16_digit<G, P>(a, tw, c, tid, T);      // t = 1024 .. 128
    group_sync(bar, G);
    fwd_passR<G, 4, P>(a, tw, c, tid, 64, 16);    // t = 64 .. 8
    group_sync(bar, G);
    fwd_passR<G, 3, P>(a, tw, c, tid, 4, 256);    // t = 4, 2, 1
    group_sync(bar, G);
}

// One radix-8 inverse pass: stages t, 2t, 4t (m = N / 2t) on the octets
// e0 + k t (k < 8) of every 8t-block.
template <int G, bool P>
__device__ __forceinline__ void inv_pass8(uint64_t *a, const ulonglong2 *__restrict__ itw, const Ntt64Consts &c,
                                          int tid, int t, int m)
{
    for (int oc = tid; oc < 256; oc += G) {
        const int grp = oc / t, j = oc - grp * t;
        const int e0 = grp * 8 * t + j;
        uint64_t x[8];
#pragma unroll
        for (int k = 0; k < 8; k++) x[k] = a[pi<P>(e0 + k * t)];
#pragma unroll
        for (int k = 0; k < 4; k++) gs64(x[2 * k], x[2 * k + 1], __ldg(itw + m + 4 * grp + k), c.Q, c.twoQ);
        const ulonglong2 w2a = __ldg(itw + (m >> 1) + 2 * grp), w2b = __ldg(itw + (m >> 1) + 2 * grp + 1);
        gs64(x[0], x[2], w2a, c.Q, c.twoQ);
        gs64(x[1], x[3], w2a, c.Q, c.twoQ);
        gs64(x[4], x[6], w2b, c.Q, c.twoQ);
        gs64(x[5], x[7], w2b, c.Q, c.twoQ);
        const ulonglong2 w4 = __ldg(itw + (m >> 2) + grp);
        gs64(x[0], x[4], w4, c.Q, c.twoQ);
        gs64(x[1], x[5], w4, c.Q, c.twoQ);
        gs64(x[2], x[6], w4, c.Q, c.twoQ);
        gs64(x[3], x[7], w4, c.Q, c.twoQ);
#pragma unroll
        for (int k = 0; k < 8; k++) a[pi<P>(e0 + k * t)] = x[k];
    }
}

// Inverse NTT of a[poly_words64<P>()] (layout pi<P>; values < 2Q, bit-reversed order) in shared memory
// -> canonical coefficients times N^-1. itw[k] = (psi^-bitrev(k), companion).
// Three radix-8 passes (stages t = 1..4, 8..32, 64..256) and one radix-4 pass
// (t = 512 and the last stage, t = 1024, with N^-1 folded into both outputs).
template <int G, bool P>
__device__ __forceinline__ void ntt64_inv_2048(uint64_t *a, const ulonglong2 *__restrict__ itw, const Ntt64Consts &c,
                                               int tid, int bar)
{
    inv_pass8<G, P>(a, itw, c, tid, 1, 1024);
    group_sync(bar, G);
    inv_pass8<G, P>(a, itw, c, tid, 8, 128);
    group_sync(bar, G);
    inv_pass8<G, P>(a, itw, c, tid, 64, 16);
    group_sync(bar, G);
    for (int b = tid; b < 512; b += G) {
        uint64_t x0 = a[pi<P>(b)], x1 = a[pi<P>(b + 512)], x2 = a[pi<P>(b + 1024)], x3 = a[pi<P>(b + 1536)];
        gs64(x0, x1, __ldg(itw + 2), c.Q, c.twoQ);   // t = 512, m = 2, block 0
        gs64(x2, x3, __ldg(itw + 3), c.Q, c.twoQ);   // block 1
        // t = 1024, m = 1, with N^-1 folded into both outputs
        uint64_t u = shoup64(x0 + x2, c.iN, c.iNs, c.Q);
        uint64_t v = shoup64(x0 - x2 + c.twoQ, c.iw1N, c.iw1Ns, c.Q);
        a[pi<P>(b)] = u >= c.Q ? u - c.Q : u;
        a[pi<P>(b + 1024)] = v >= c.Q ? v - c.Q : v;
        u = shoup64(x1 + x3, c.iN, c.iNs, c.Q);
        v = shoup64(x1 - x3 + c.twoQ, c.iw1N, c.iw1Ns, c.Q);
        a[pi<P>(b + 512)] = u >= c.Q ? u - c.Q : u;
        a[pi<P>(b + 1536)] = v >= c.Q ? v - c.Q : v;
    }
    group_sync(bar, G);
}

}  // namespace dev
}  // namespace fheacc
