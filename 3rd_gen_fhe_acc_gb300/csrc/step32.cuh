// step32.cuh -- shared pieces of the 32-bit RLWE x RGSW step: Barrett
// reductions, key readers, and the three-phase step on a CTA-resident
// accumulator used by the stand-alone RLWE x RGSW entry point.
// Reference: RLWE_mult_RGSW (FHE_ACC_runtime/src/RLWE.cpp:642-704) and
// digit_decompose (RLWE.cpp:623-640).
#pragma once
#include "l2hint.cuh"
#include "ntt32.cuh"

namespace fheacc {
namespace dev {

// floor(x / Q) estimate error of at most one: result in [0, 2Q).
__device__ __forceinline__ uint32_t barrett64_lazy(uint64_t s, uint64_t mu64, uint32_t Q)
{
    uint64_t qe = __umul64hi(s, mu64);
    return (uint32_t)s - (uint32_t)qe * Q;
}

// x < 2^32 -> canonical, mu32 = floor(2^32 / Q)
__device__ __forceinline__ uint32_t reduce32(uint32_t x, uint32_t mu32, uint32_t Q)
{
    uint32_t r = x - __umulhi(x, mu32) * Q;
    return min(r, r - Q);
}

// Montgomery reduction of a multiply-accumulate sum s < 2^62: s 2^-32 mod Q
// in [0, 2Q). The sum of 2 digitG products (NTT digits < 21Q, keys < Q) is
// below 168 Q^2, so (s + m Q) / 2^32 < 6.25 Q before the two conditional
// subtractions.
__device__ __forceinline__ uint32_t mont_reduce_2q(uint64_t s, uint32_t Q, uint32_t qinv_neg)
{
    const uint32_t m = (uint32_t)s * qinv_neg;
    uint32_t r = (uint32_t)((s + (uint64_t)m * Q) >> 32);
    r = min(r, r - 4 * Q);
    return min(r, r - 2 * Q);
}

// Multiply-accumulate of one 4-element chunk u (elements 32 (u % 32) + 4 (u / 32)
// + 0..3 of both output polys): acc[P][e] = sum over (p, h) of dbuf[p][h][e] *
// key[h][p][P][e], Montgomery-reduced. With acc_nd (the item's NTT-domain
// accumulator, B-tiled, read before it is overwritten) the last digit's term
// uses acc_nd[p] in place of its NTT (keys uploaded for that identity).
// KEEP: the accumulator is read and written with the L2 evict-last policy
// (l2hint.cuh), for accumulators that the next step reads again.
template <int DG, bool DERIVE = false, bool KEEP = false>
__device__ __forceinline__ void mac_chunk(int u, const uint4 *__restrict__ key,
                                          const uint32_t (*dbuf)[kN32], uint4 *acc, uint32_t Q, uint32_t qinv_neg,
                                          const uint4 *acc_nd = nullptr)
{
    constexpr int DT = DERIVE ? DG - 1 : DG;   // digit NTTs per poly in dbuf: [p * DT + h]
    const int pa = sw_chunk(u & 31, u >> 5);
    const uint64_t pol = KEEP ? l2_keep_policy() : 0;
    uint64_t sa[4] = {0, 0, 0, 0}, sb[4] = {0, 0, 0, 0};
#pragma unroll
    for (int qi = 0; qi < 2 * DG; qi++) {
        const int pp = qi / DG, hh = qi % DG;
        const uint4 dv = (DERIVE && hh == DG - 1)
                             ? (KEEP ? ld_keep(acc_nd + pp * 256 + u, pol) : __ldcg(acc_nd + pp * 256 + u))
                             : *reinterpret_cast<const uint4 *>(dbuf[pp * DT + hh] + pa);
        // keys stream through L2 only: an item's 64 KB would otherwise evict
        // the transforms' twiddle tables from the L1 left beside shared memory
        const uint4 a4 = __ldcg(key + ((hh * 2 + pp) * 2 + 0) * 256 + u);
        const uint4 b4 = __ldcg(key + ((hh * 2 + pp) * 2 + 1) * 256 + u);
        sa[0] += (uint64_t)dv.x * a4.x; sb[0] += (uint64_t)dv.x * b4.x;
        sa[1] += (uint64_t)dv.y * a4.y; sb[1] += (uint64_t)dv.y * b4.y;
        sa[2] += (uint64_t)dv.z * a4.z; sb[2] += (uint64_t)dv.z * b4.z;
        sa[3] += (uint64_t)dv.w * a4.w; sb[3] += (uint64_t)dv.w * b4.w;
    }
    const uint4 ra = make_uint4(mont_reduce_2q(sa[0], Q, qinv_neg), mont_reduce_2q(sa[1], Q, qinv_neg),
                                mont_reduce_2q(sa[2], Q, qinv_neg), mont_reduce_2q(sa[3], Q, qinv_neg));
    const uint4 rb = make_uint4(mont_reduce_2q(sb[0], Q, qinv_neg), mont_reduce_2q(sb[1], Q, qinv_neg),
                                mont_reduce_2q(sb[2], Q, qinv_neg), mont_reduce_2q(sb[3], Q, qinv_neg));
    if (KEEP) {
        st_keep(acc + u, ra, pol);
        st_keep(acc + 256 + u, rb, pol);
    } else {
        __stcg(acc + u, ra);
        __stcg(acc + 256 + u, rb);
    }
}

// Shared-memory working set of one CTA.
template <int DG>
struct StepSmem {
    uint32_t acc[2][kPadN];        // NTT-domain accumulator, values < 2Q
    uint32_t tbuf[2][kPadN];       // time-domain accumulator, canonical
    uint32_t dbuf[2 * DG][kPadN];  // digit NTTs / per-warp transpose scratch
};

// Phase 1: warps 0 and 1 move acc to the time domain. `reverse_a` applies the
// reference's NTT_a_transpose (RLWE.cpp:218-226) to poly a first.
template <int DG>
__device__ __forceinline__ void phase_intt(StepSmem<DG> &s, const Ntt32Consts &c, const uint2 *inv_tw, int warp,
                                           int lane, bool reverse_a)
{
    if (warp < 2) {
        uint32_t x[32];
        const uint32_t *src = s.acc[warp];
        if (warp == 0 && reverse_a) {
#pragma unroll
            for (int r = 0; r < 32; r++) x[r] = src[33 * (31 - lane) + (31 - r)];
        } else {
#pragma unroll
            for (int r = 0; r < 32; r++) x[r] = src[33 * lane + r];
        }
        ntt_inv_1024(x, c, inv_tw, s.dbuf[warp], lane);
#pragma unroll
        for (int r = 0; r < 32; r++) s.tbuf[warp][33 * r + lane] = x[r];
    }
}

// Phase 2: warp w = p * DG + h decomposes poly p into digit h and transforms it.
template <int DG>
__device__ __forceinline__ void phase_digits(StepSmem<DG> &s, const Ntt32Consts &c, const uint2 *fwd_tw, int warp,
                                             int lane, uint32_t bg_bits)
{
    if (warp < 2 * DG) {
        const int p = warp / DG, h = warp % DG;
        const uint32_t shift = bg_bits * h, mask = (1u << bg_bits) - 1;
        uint32_t x[32];
#pragma unroll
        for (int r = 0; r < 32; r++) x[r] = (s.tbuf[p][33 * r + lane] >> shift) & mask;
        ntt_fwd_1024(x, c, fwd_tw, s.dbuf[warp], lane);
#pragma unroll
        for (int r = 0; r < 32; r++) s.dbuf[warp][33 * lane + r] = x[r];
    }
}

// Key row reader over the device layout [h][g][P][N] (u32).
struct KeyU32 {
    const uint32_t *base;
    __device__ __forceinline__ uint4 load4(int h, int g, int P, int k) const
    {
        return __ldg(reinterpret_cast<const uint4 *>(base + (((h * 2 + g) * 2 + P) << 10) + k));
    }
};

// Key row reader over the reference layout c_text[h][g].{a,b}[k] (u64).
struct KeyU64Ref {
    const uint64_t *base;
    __device__ __forceinline__ uint4 load4(int h, int g, int P, int k) const
    {
        const uint64_t *p = base + (((h * 2 + g) * 2 + P) << 10) + k;
        return make_uint4((uint32_t)p[0], (uint32_t)p[1], (uint32_t)p[2], (uint32_t)p[3]);
    }
};

// Phase 3: multiply-accumulate with the RGSW key, write acc (values < 2Q).
template <int DG, class Key>
__device__ __forceinline__ void phase_mac(StepSmem<DG> &s, const Key &key, uint64_t mu64, uint32_t Q)
{
    for (int t = threadIdx.x; t < 256; t += blockDim.x) {
        const int k0 = 4 * t;
        const int pa = k0 + (k0 >> 5);   // the 4 words of a quad share k0 >> 5
        uint64_t sa[4] = {0, 0, 0, 0}, sb[4] = {0, 0, 0, 0};
#pragma unroll
        for (int p = 0; p < 2; p++) {
#pragma unroll
            for (int h = 0; h < DG; h++) {
                const uint32_t *d = s.dbuf[p * DG + h] + pa;
                const uint4 ka = key.load4(h, p, 0, k0);
                const uint4 kb = key.load4(h, p, 1, k0);
                const uint32_t d0 = d[0], d1 = d[1], d2 = d[2], d3 = d[3];
                sa[0] += (uint64_t)d0 * ka.x; sb[0] += (uint64_t)d0 * kb.x;
                sa[1] += (uint64_t)d1 * ka.y; sb[1] += (uint64_t)d1 * kb.y;
                sa[2] += (uint64_t)d2 * ka.z; sb[2] += (uint64_t)d2 * kb.z;
                sa[3] += (uint64_t)d3 * ka.w; sb[3] += (uint64_t)d3 * kb.w;
            }
        }
#pragma unroll
        for (int e = 0; e < 4; e++) {
            s.acc[0][pa + e] = barrett64_lazy(sa[e], mu64, Q);
            s.acc[1][pa + e] = barrett64_lazy(sb[e], mu64, Q);
        }
    }
}

// One RLWE x RGSW step on the CTA's accumulator in shared memory.
template <int DG, class Key>
__device__ __forceinline__ void rlwe_x_rgsw_step(StepSmem<DG> &s, const Ntt32Consts &c, const uint2 *fwd_tw,
                                                 const uint2 *inv_tw, const Key &key, uint32_t bg_bits,
                                                 uint64_t mu64, int warp, int lane)
{
    phase_intt<DG>(s, c, inv_tw, warp, lane, false);
    __syncthreads();
    phase_digits<DG>(s, c, fwd_tw, warp, lane, bg_bits);
    __syncthreads();
    phase_mac<DG>(s, key, mu64, c.Q);
    __syncthreads();
}

}  // namespace dev
}  // namespace fheacc
