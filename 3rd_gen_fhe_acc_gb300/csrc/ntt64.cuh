// ntt64.cuh -- negacyclic NTT / inverse NTT of a 2048-point polynomial with
// 64-bit words (Q < 2^62), computed in shared memory by a group of threads.
//
// Same transforms as the reference's NTT / iNTT (FHE_ACC_runtime/src/
// nbt.cpp:423-454 and 456-491), so canonical outputs are bit-identical.
//
// A 64-bit Shoup multiplication (w' = floor(w 2^64 / Q)) costs about five
// times a 32-bit one, so shared-memory traffic matters less here than in the
// 32-bit path: the polynomial stays in shared memory and each thread runs
// radix-4 passes (two butterfly stages per load/store of four words), with one
// group barrier per pass. Forward butterflies leave the upper input unreduced
// (bound grows by 2Q a stage: inputs < Q end below 23Q < 2^59 for Q < 2^54);
// the inverse keeps Harvey's [0, 2Q) invariant and ends canonical.
#pragma once
#include <cstdint>

namespace fheacc {
namespace dev {

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

// Forward NTT of a[2048] in shared memory by `G` threads (tid < G) that share
// the named barrier `bar`. tw[k] = (psi^bitrev(k), companion). Input < Q,
// output < 23Q, bit-reversed order as the reference's.
template <int G>
__device__ __forceinline__ void ntt64_fwd_2048(uint64_t *a, const ulonglong2 *__restrict__ tw, const Ntt64Consts &c,
                                               int tid, int bar)
{
    constexpr int N = 2048;
    int m = 1;
#pragma unroll 1
    for (int t = N / 2; t >= 2; t >>= 2, m <<= 2) {   // stages (t, t/2)
        const int h = t >> 1;
        for (int qd = tid; qd < N / 4; qd += G) {
            const int grp = qd / h, j = qd - grp * h;
            const int e0 = grp * 2 * t + j;
            uint64_t x0 = a[e0], x1 = a[e0 + h], x2 = a[e0 + t], x3 = a[e0 + t + h];
            const ulonglong2 w = __ldg(tw + m + grp);
            ct64(x0, x2, w, c.Q, c.twoQ);
            ct64(x1, x3, w, c.Q, c.twoQ);
            ct64(x0, x1, __ldg(tw + 2 * m + 2 * grp), c.Q, c.twoQ);
            ct64(x2, x3, __ldg(tw + 2 * m + 2 * grp + 1), c.Q, c.twoQ);
            a[e0] = x0; a[e0 + h] = x1; a[e0 + t] = x2; a[e0 + t + h] = x3;
        }
        group_sync(bar, G);
    }
    // last stage, t = 1, m = 1024
    for (int b = tid; b < N / 2; b += G) {
        uint64_t x = a[2 * b], y = a[2 * b + 1];
        ct64(x, y, __ldg(tw + 1024 + b), c.Q, c.twoQ);
        a[2 * b] = x;
        a[2 * b + 1] = y;
    }
    group_sync(bar, G);
}

// Inverse NTT of a[2048] (values < 2Q, bit-reversed order) in shared memory
// -> canonical coefficients times N^-1. itw[k] = (psi^-bitrev(k), companion).
template <int G>
__device__ __forceinline__ void ntt64_inv_2048(uint64_t *a, const ulonglong2 *__restrict__ itw, const Ntt64Consts &c,
                                               int tid, int bar)
{
    constexpr int N = 2048;
    int m = N / 2;
#pragma unroll 1
    for (int t = 1; t <= N / 8; t <<= 2, m >>= 2) {   // stages (t, 2t)
        for (int qd = tid; qd < N / 4; qd += G) {
            const int grp = qd / t, j = qd - grp * t;
            const int e0 = grp * 4 * t + j;
            uint64_t x0 = a[e0], x1 = a[e0 + t], x2 = a[e0 + 2 * t], x3 = a[e0 + 3 * t];
            gs64(x0, x1, __ldg(itw + m + 2 * grp), c.Q, c.twoQ);
            gs64(x2, x3, __ldg(itw + m + 2 * grp + 1), c.Q, c.twoQ);
            const ulonglong2 w = __ldg(itw + (m >> 1) + grp);
            gs64(x0, x2, w, c.Q, c.twoQ);
            gs64(x1, x3, w, c.Q, c.twoQ);
            a[e0] = x0; a[e0 + t] = x1; a[e0 + 2 * t] = x2; a[e0 + 3 * t] = x3;
        }
        group_sync(bar, G);
    }
    // last stage, t = 1024, m = 1, with N^-1 folded into both outputs
    for (int b = tid; b < N / 2; b += G) {
        const uint64_t x = a[b], y = a[b + 1024];
        uint64_t u = shoup64(x + y, c.iN, c.iNs, c.Q);
        uint64_t v = shoup64(x - y + c.twoQ, c.iw1N, c.iw1Ns, c.Q);
        a[b] = u >= c.Q ? u - c.Q : u;
        a[b + 1024] = v >= c.Q ? v - c.Q : v;
    }
    group_sync(bar, G);
}

}  // namespace dev
}  // namespace fheacc
