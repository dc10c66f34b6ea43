// expand.cu -- the X -> X^k automorphism, the RLWE key switch and
// expand_RLWE, for both word widths.
//
// Reference behaviour: RLWE_substitute (FHE_ACC_runtime/src/RLWE.cpp:444-462)
// with poly_substitute (RLWE.cpp:23-37), RLWE_keyswitch (RLWE.cpp:464-510),
// RLWE_rotate_freq (RLWE.cpp:411-430) and application::expand_RLWE
// (app.cpp:26-76); on the FPGA the RLWESUBS instruction (subs_module.sv +
// the NTT/MAC chain) and fpga_expand_RLWE (myfpga.cpp:1662-1790).
//
// One CTA handles one RLWE (an "item"). The substitution is applied while the
// time-domain coefficients are read: out[e] = in[i'] when i' < N, else
// -in[i' - N], with i' = e * power^-1 mod 2N and power = N / 2^f + 1 (odd) --
// the inverse of poly_substitute's scatter out[i * power mod N] = +-in[i]. The
// key switch then decomposes sigma(a) in base 2^Bks_R_bits, transforms each
// digit and multiply-accumulates with the key rows; sigma(b) is transformed
// once. Modes:
//   SUBS      out = RLWE_substitute(c, f)
//   KS        out = RLWE_keyswitch(c, ksk)                (f = 0 is the identity)
//   SUBS_KS   out = RLWE_keyswitch(RLWE_substitute(c, f), ksk)
//   EXPAND    r[j] <- r[j] + s, r[j + 2^f] <- (r[j] - s) * NTT(-X^(N - 2^f)),
//             s = SUBS_KS(r[j], f, subs_key[f]), for every j < 2^f (one level)
#include "ctx.hpp"
#include "step32.cuh"
#include <algorithm>

namespace fheacc {
namespace dev {

enum ExpMode { kSubs = 0, kKs = 1, kSubsKs = 2, kExpand = 3 };

struct ExpArgs {
    const uint64_t *in;      // items [count][2N] (EXPAND: the r arrays)
    uint64_t *out;           // [count][2N] (EXPAND: the r arrays, in place)
    size_t count;
    size_t batches;          // EXPAND: independent r arrays, bstride words apart (else 1)
    size_t bstride;
    int mode, f, logN, L;    // L = digitKS_R
    uint32_t bits;           // Bks_R_bits
    uint32_t ipow;           // (N / 2^f + 1)^-1 mod 2N
    const uint32_t *ksk32;   // [L][2][N] u32 (narrow)
    const ulonglong2 *ksk64; // [L][2][N] Shoup pairs (wide)
    const uint64_t *rot;     // [N] NTT(-X^(N - 2^f)) (EXPAND)
    uint64_t Q, mu64;
};

__device__ __forceinline__ uint32_t subs_src(uint32_t e, uint32_t ipow, uint32_t N, bool &neg)
{
    const uint32_t ip = (uint32_t)(((uint64_t)e * ipow) & (2 * N - 1));
    neg = ip >= N;
    return neg ? ip - N : ip;
}

// ---------------------------------------------------------------- narrow
// 8 warps: warps 0/1 inverse NTTs, then warps 0..L-1 the digits of sigma(a)
// and warp L sigma(b), then all threads the MAC and the epilogue.
__global__ void __launch_bounds__(256) expand32_kernel(const __grid_constant__ ExpArgs A,
                                                      const __grid_constant__ Ntt32Consts c,
                                                      const uint2 *__restrict__ fwd_tw,
                                                      const uint2 *__restrict__ inv_tw, uint32_t mu32)
{
    __shared__ __align__(16) uint32_t t[2][kPadN];
    __shared__ __align__(16) uint32_t d[5][kPadN];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t Q = c.Q;
    const int L = A.L;
    const bool subs = A.mode != kKs;
    const size_t per = A.mode == kExpand ? ((size_t)1 << A.f) : A.count;
    const size_t items = per * A.batches;
    for (size_t it = blockIdx.x; it < items; it += gridDim.x) {
        const size_t bo = it / per * A.bstride, jt = it % per;   // batch offset, item within the batch
        const uint64_t *in = A.in + bo + jt * 2048;
        if (warp < 2) {
            uint32_t x[32];
#pragma unroll
            for (int r = 0; r < 32; r++) x[r] = (uint32_t)in[warp * 1024 + 32 * lane + r];
            ntt_inv_1024(x, c, inv_tw, d[warp], lane);
#pragma unroll
            for (int r = 0; r < 32; r++) t[warp][pad32(lane + 32 * r)] = x[r];
        }
        __syncthreads();
        const int nt = A.mode == kSubs ? 2 : L + 1;   // transforms of phase 2
        if (warp < nt) {
            // kSubs: warps 0, 1 transform sigma(a), sigma(b); else warps < L
            // the digits of sigma(a) and warp L sigma(b)
            const int poly = A.mode == kSubs ? warp : (warp == L ? 1 : 0);
            const bool digit = A.mode != kSubs && warp < L;
            const uint32_t sh = A.bits * (uint32_t)warp, mask = (1u << A.bits) - 1;
            uint32_t x[32];
#pragma unroll
            for (int r = 0; r < 32; r++) {
                const uint32_t e = lane + 32 * r;
                uint32_t v;
                if (subs) {
                    bool neg;
                    const uint32_t s = subs_src(e, A.ipow, 1024, neg);
                    v = t[poly][pad32(s)];
                    if (neg && v) v = Q - v;
                } else {
                    v = t[poly][pad32(e)];
                }
                x[r] = digit ? (v >> sh) & mask : v;
            }
            ntt_fwd_1024(x, c, fwd_tw, d[warp], lane);
#pragma unroll
            for (int r = 0; r < 32; r++) d[warp][33 * lane + r] = reduce32(x[r], mu32, Q);
        }
        __syncthreads();
        uint64_t *out = A.out + bo + jt * 2048;
        for (int k = threadIdx.x; k < 1024; k += blockDim.x) {
            uint64_t oa, ob;
            if (A.mode == kSubs) {
                oa = d[0][pad32(k)];
                ob = d[1][pad32(k)];
            } else {
                uint64_t sa = 0, sb = 0;
                for (int h = 0; h < L; h++) {
                    const uint64_t dv = d[h][pad32(k)];
                    sa += dv * A.ksk32[(h * 2 + 0) * 1024 + k];
                    sb += dv * A.ksk32[(h * 2 + 1) * 1024 + k];
                }
                const uint32_t ra = barrett64_lazy(sa, A.mu64, Q), rb = barrett64_lazy(sb, A.mu64, Q);
                const uint32_t ca = min(ra, ra - Q), cb = min(rb, rb - Q);
                oa = ca ? Q - ca : 0;
                const uint32_t nb = d[L][pad32(k)];
                ob = nb >= cb ? nb - cb : nb + Q - cb;
            }
            if (A.mode == kExpand) {
                const uint64_t ta = in[k], tb = in[1024 + k];
                const uint64_t rot = A.rot[k];
                uint64_t *hi = A.out + bo + (jt + per) * 2048;
                out[k] = (ta + oa) % Q;
                out[1024 + k] = (tb + ob) % Q;
                hi[k] = ((ta + Q - oa) % Q) * rot % Q;
                hi[1024 + k] = ((tb + Q - ob) % Q) * rot % Q;
            } else {
                out[k] = oa;
                out[1024 + k] = ob;
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------- wide
// 256 threads in two 128-thread groups; group g transforms poly g.
__global__ void __launch_bounds__(256) expand64_kernel(const __grid_constant__ ExpArgs A,
                                                      const ulonglong2 *__restrict__ tw,
                                                      const ulonglong2 *__restrict__ itw,
                                                      const __grid_constant__ Ntt64Consts c)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint64_t(*t)[2048] = reinterpret_cast<uint64_t(*)[2048]>(smem_raw);                 // [2][2048]
    uint64_t(*buf)[2048] = reinterpret_cast<uint64_t(*)[2048]>(smem_raw + 2 * 2048 * 8);  // [2][2048]
    const int tid = threadIdx.x, grp = tid >> 7, gtid = tid & 127;
    const uint64_t Q = c.Q;
    const int L = A.L;
    const bool subs = A.mode != kKs;
    const size_t per = A.mode == kExpand ? ((size_t)1 << A.f) : A.count;
    const size_t items = per * A.batches;
    for (size_t it = blockIdx.x; it < items; it += gridDim.x) {
        const size_t bo = it / per * A.bstride, jt = it % per;   // batch offset, item within the batch
        const uint64_t *in = A.in + bo + jt * 4096;
        for (int e = gtid; e < 2048; e += 128) t[grp][e] = in[grp * 2048 + e];
        group_sync(1 + grp, 128);
        ntt64_inv_2048<128, false>(t[grp], itw, c, gtid, 1 + grp);
        __syncthreads();
        // transforms: L digits of sigma(a) and sigma(b) (SUBS: sigma(a), sigma(b)),
        // two at a time; MAC after each pair
        const int nt = A.mode == kSubs ? 2 : L + 1;
        uint64_t sa[8], sb[8], fb[8];
#pragma unroll
        for (int i = 0; i < 8; i++) sa[i] = sb[i] = fb[i] = 0;
        for (int base = 0; base < nt; base += 2) {
            const int tr = base + grp;   // transform index of this group
            if (tr < nt) {
                const int poly = A.mode == kSubs ? tr : (tr == L ? 1 : 0);
                const bool digit = A.mode != kSubs && tr < L;
                const uint32_t sh = A.bits * (uint32_t)tr;
                const uint64_t mask = (1ULL << A.bits) - 1;
                for (int e = gtid; e < 2048; e += 128) {
                    uint64_t v;
                    if (subs) {
                        bool neg;
                        const uint32_t s = subs_src((uint32_t)e, A.ipow, 2048, neg);
                        v = t[poly][s];
                        if (neg && v) v = Q - v;
                    } else {
                        v = t[poly][e];
                    }
                    buf[grp][e] = digit ? (v >> sh) & mask : v;
                }
                group_sync(1 + grp, 128);
                ntt64_fwd_2048<128, false>(buf[grp], tw, c, gtid, 1 + grp);
            }
            __syncthreads();
#pragma unroll
            for (int i = 0; i < 8; i++) {
                const int k = tid + 256 * i;
#pragma unroll
                for (int g2 = 0; g2 < 2; g2++) {
                    const int tr = base + g2;
                    if (tr >= nt) continue;
                    const uint64_t dv = buf[g2][k];
                    if (A.mode == kSubs || tr == L) {
                        const uint64_t v = barrett64_2q(dv, c.mu64, Q);
                        if (A.mode == kSubs && tr == 0) sa[i] = v;
                        else fb[i] = v;
                    } else {
                        const ulonglong2 ka = __ldg(A.ksk64 + (size_t)(tr * 2 + 0) * 2048 + k);
                        const ulonglong2 kb = __ldg(A.ksk64 + (size_t)(tr * 2 + 1) * 2048 + k);
                        sa[i] += shoup64(dv, ka.x, ka.y, Q);
                        sb[i] += shoup64(dv, kb.x, kb.y, Q);
                    }
                }
            }
            __syncthreads();
        }
        uint64_t *out = A.out + bo + jt * 4096;
#pragma unroll
        for (int i = 0; i < 8; i++) {
            const int k = tid + 256 * i;
            uint64_t oa, ob;
            if (A.mode == kSubs) {
                oa = sa[i] >= Q ? sa[i] - Q : sa[i];
                ob = fb[i] >= Q ? fb[i] - Q : fb[i];
            } else {
                uint64_t ra = barrett64_2q(sa[i], c.mu64, Q), rb = barrett64_2q(sb[i], c.mu64, Q);
                ra = ra >= Q ? ra - Q : ra;
                rb = rb >= Q ? rb - Q : rb;
                const uint64_t nb = fb[i] >= Q ? fb[i] - Q : fb[i];
                oa = ra ? Q - ra : 0;
                ob = nb >= rb ? nb - rb : nb + Q - rb;
            }
            if (A.mode == kExpand) {
                const uint64_t ta = in[k], tb = in[2048 + k];
                const uint64_t rot = A.rot[k];
                uint64_t *hi = A.out + bo + (jt + per) * 4096;
                const uint64_t s1 = ta + oa, s2 = tb + ob;
                out[k] = s1 >= Q ? s1 - Q : s1;
                out[2048 + k] = s2 >= Q ? s2 - Q : s2;
                const uint64_t d1 = ta >= oa ? ta - oa : ta + Q - oa, d2 = tb >= ob ? tb - ob : tb + Q - ob;
                hi[k] = (uint64_t)((unsigned __int128)d1 * rot % Q);
                hi[2048 + k] = (uint64_t)((unsigned __int128)d2 * rot % Q);
            } else {
                out[k] = oa;
                out[2048 + k] = ob;
            }
        }
        __syncthreads();
    }
}

// An expand_RLWE level of few RLWEs (64-bit words), split over the transform
// pairs for latency: CTA (item, pair p) takes the item's inverse NTTs, transforms
// 2p and 2p + 1 of the L + 1 (the key-switch digits of sigma(a), transform L
// sigma(b)) and their share of the key multiply-accumulate, written to
// part[item][p] as [sa | sb | fb][2048], each word < 4Q. expand64_combine_kernel
// adds the shares and applies the level's epilogue. One RLWE's transforms then
// take two rounds instead of 1 + ceil((L + 1) / 2).
__global__ void __launch_bounds__(256) expand64_split_kernel(const __grid_constant__ ExpArgs A,
                                                            uint64_t *__restrict__ part, int P,
                                                            const ulonglong2 *__restrict__ tw,
                                                            const ulonglong2 *__restrict__ itw,
                                                            const __grid_constant__ Ntt64Consts c)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint64_t(*t)[2048] = reinterpret_cast<uint64_t(*)[2048]>(smem_raw);                 // [2][2048]
    uint64_t(*buf)[2048] = reinterpret_cast<uint64_t(*)[2048]>(smem_raw + 2 * 2048 * 8);  // [2][2048]
    const int tid = threadIdx.x, grp = tid >> 7, gtid = tid & 127;
    const uint64_t Q = c.Q;
    const int L = A.L, nt = L + 1;
    const size_t per = (size_t)1 << A.f;
    const size_t it = blockIdx.x / (unsigned)P;
    const int p = (int)(blockIdx.x - it * (unsigned)P);
    const size_t bo = it / per * A.bstride, jt = it % per;
    const uint64_t *in = A.in + bo + jt * 4096;
    for (int e = gtid; e < 2048; e += 128) t[grp][e] = in[grp * 2048 + e];
    group_sync(1 + grp, 128);
    ntt64_inv_2048<128, false>(t[grp], itw, c, gtid, 1 + grp);
    __syncthreads();
    const int tr = 2 * p + grp;
    if (tr < nt) {
        const int poly = tr == L ? 1 : 0;
        const bool digit = tr < L;
        const uint32_t sh = A.bits * (uint32_t)tr;
        const uint64_t mask = (1ULL << A.bits) - 1;
        for (int e = gtid; e < 2048; e += 128) {
            bool neg;
            const uint32_t s = subs_src((uint32_t)e, A.ipow, 2048, neg);
            uint64_t v = t[poly][s];
            if (neg && v) v = Q - v;
            buf[grp][e] = digit ? (v >> sh) & mask : v;
        }
        group_sync(1 + grp, 128);
        ntt64_fwd_2048<128, false>(buf[grp], tw, c, gtid, 1 + grp);
    }
    __syncthreads();
    uint64_t *o = part + (it * (unsigned)P + (unsigned)p) * 3 * 2048;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int k = tid + 256 * i;
        uint64_t sa = 0, sb = 0, fb = 0;
#pragma unroll
        for (int g2 = 0; g2 < 2; g2++) {
            const int tq = 2 * p + g2;
            if (tq >= nt) continue;
            const uint64_t dv = buf[g2][k];
            if (tq == L) {
                fb = barrett64_2q(dv, c.mu64, Q);
            } else {
                const ulonglong2 ka = __ldg(A.ksk64 + (size_t)(tq * 2 + 0) * 2048 + k);
                const ulonglong2 kb = __ldg(A.ksk64 + (size_t)(tq * 2 + 1) * 2048 + k);
                sa += shoup64(dv, ka.x, ka.y, Q);
                sb += shoup64(dv, kb.x, kb.y, Q);
            }
        }
        o[k] = sa;
        o[2048 + k] = sb;
        o[4096 + k] = fb;
    }
}

// The shares of expand64_split_kernel added (P of them, < 4PQ < 2^64, checked
// by the launcher) and the expand level's epilogue, one thread per item word:
// s = (-sa, sigma(b) - sb), r[j] <- r[j] + s, r[j + 2^f] <- (r[j] - s) * rot.
__global__ void expand64_combine_kernel(const __grid_constant__ ExpArgs A, const uint64_t *__restrict__ part, int P,
                                        size_t items, const __grid_constant__ Ntt64Consts c)
{
    const uint64_t Q = c.Q;
    const size_t per = (size_t)1 << A.f;
    for (size_t w = (size_t)blockIdx.x * blockDim.x + threadIdx.x; w < items * 2048;
         w += (size_t)gridDim.x * blockDim.x) {
        const size_t it = w / 2048;
        const int k = (int)(w - it * 2048);
        const size_t bo = it / per * A.bstride, jt = it % per;
        const uint64_t *pp = part + it * (unsigned)P * 3 * 2048 + k;
        uint64_t sa = 0, sb = 0, fb = 0;
        for (int p = 0; p < P; p++) {
            sa += pp[(size_t)(p * 3 + 0) * 2048];
            sb += pp[(size_t)(p * 3 + 1) * 2048];
            fb += pp[(size_t)(p * 3 + 2) * 2048];
        }
        uint64_t ra = barrett64_2q(sa, c.mu64, Q), rb = barrett64_2q(sb, c.mu64, Q);
        ra = ra >= Q ? ra - Q : ra;
        rb = rb >= Q ? rb - Q : rb;
        const uint64_t nb = fb >= Q ? fb - Q : fb;
        const uint64_t oa = ra ? Q - ra : 0;
        const uint64_t ob = nb >= rb ? nb - rb : nb + Q - rb;
        const uint64_t *in = A.in + bo + jt * 4096;
        uint64_t *out = A.out + bo + jt * 4096;
        uint64_t *hi = A.out + bo + (jt + per) * 4096;
        const uint64_t ta = in[k], tb = in[2048 + k];
        const uint64_t rot = A.rot[k];
        const uint64_t s1 = ta + oa, s2 = tb + ob;
        out[k] = s1 >= Q ? s1 - Q : s1;
        out[2048 + k] = s2 >= Q ? s2 - Q : s2;
        const uint64_t d1 = ta >= oa ? ta - oa : ta + Q - oa, d2 = tb >= ob ? tb - ob : tb + Q - ob;
        hi[k] = (uint64_t)((unsigned __int128)d1 * rot % Q);
        hi[2048 + k] = (uint64_t)((unsigned __int128)d2 * rot % Q);
    }
}

__global__ void to_u32_kernel(const uint64_t *__restrict__ in, uint32_t *__restrict__ out, size_t n, uint64_t Q)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = (uint32_t)(in[i] % Q);
}

}  // namespace dev

static int sms(Context &c)
{
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, c.device);
    return v > 0 ? v : 1;
}

static uint32_t inv_power(int N, int f)
{
    const uint64_t m = 2ULL * (uint64_t)N, p = (uint64_t)(N >> f) + 1;
    for (uint64_t x = 1; x < m; x += 2)
        if ((x * p) % m == 1) return (uint32_t)x;
    return 1;
}

// ksk: narrow, u32 [L][2][N] device words; wide, Shoup pairs.
int launch_expand(Context &c, int mode, const uint64_t *d_in, uint64_t *d_out, size_t count, int f,
                  const void *ksk, const uint64_t *d_rot, cudaStream_t st, size_t batches, size_t bstride)
{
    const int logN = c.wide ? 11 : 10;
    if (f < 0 || f >= logN) return c.fail(FHEACC_EINVAL, "substitution factor out of range");
    dev::ExpArgs A{};
    A.in = d_in; A.out = d_out; A.count = count; A.mode = mode; A.f = f; A.logN = logN;
    A.batches = mode == dev::kExpand ? batches : 1;
    A.bstride = bstride;
    A.L = (int)c.p.digitKS_R; A.bits = c.p.Bks_R_bits; A.ipow = inv_power(c.p.N, mode == dev::kKs ? 0 : f);
    A.rot = d_rot; A.Q = c.p.Q; A.mu64 = c.dp.mu64;
    if (mode == dev::kKs) A.ipow = 1;
    const size_t items = (mode == dev::kExpand ? ((size_t)1 << f) : count) * A.batches;
    if (!items) return FHEACC_OK;
    size_t blocks = std::min<size_t>(items, (size_t)sms(c) * 4);
    cudaError_t e;
    if (c.wide) {
        if (A.L > 8) return c.fail(FHEACC_EINVAL, "digitKS_R too large");
        A.ksk64 = (const ulonglong2 *)ksk;
        const size_t smem = 4 * 2048 * sizeof(uint64_t);
        // an expand level of at most two CTAs per SM of (item, transform pair)
        // splits each item over its transform pairs, for latency
        const int P = (A.L + 2) / 2;
        if (mode == dev::kExpand && items * P <= (size_t)sms(c) * 2 && (uint64_t)4 * P < UINT64_MAX / c.p.Q) {
            const size_t words = items * P * 3 * 2048;
            int rc = ensure_scratch(c, c.expand, words * sizeof(uint64_t));
            if (rc) return rc;
            uint64_t *part = (uint64_t *)c.expand.ptr;
            cudaFuncSetAttribute(dev::expand64_split_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            dev::expand64_split_kernel<<<(unsigned)(items * P), 256, smem, st>>>(A, part, P, c.d_tw64, c.d_itw64,
                                                                                 c.nc64);
            c.launches++;
            e = cudaGetLastError();
            if (e != cudaSuccess) return c.cuda_fail(e, "expand split launch");
            const unsigned cb = (unsigned)std::min<size_t>((items * 2048 + 255) / 256, (size_t)sms(c) * 4);
            dev::expand64_combine_kernel<<<cb, 256, 0, st>>>(A, part, P, items, c.nc64);
            c.launches++;
            e = cudaGetLastError();
            return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "expand combine launch");
        }
        cudaFuncSetAttribute(dev::expand64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        dev::expand64_kernel<<<(unsigned)blocks, 256, smem, st>>>(A, c.d_tw64, c.d_itw64, c.nc64);
        c.launches++;
    } else {
        if (A.L > 4) return c.fail(FHEACC_EINVAL, "digitKS_R too large for the 32-bit path");
        A.ksk32 = (const uint32_t *)ksk;
        dev::expand32_kernel<<<(unsigned)blocks, 256, 0, st>>>(A, c.nc, c.d_fwd_tw, c.d_inv_tw,
                                                              (uint32_t)((1ULL << 32) / c.p.Q));
        c.launches++;
    }
    e = cudaGetLastError();
    return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "expand launch");
}

int launch_to_u32(Context &c, const uint64_t *d_in, uint32_t *d_out, size_t n, cudaStream_t st)
{
    if (!n) return FHEACC_OK;
    unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, (size_t)sms(c) * 32);
    dev::to_u32_kernel<<<blocks, 256, 0, st>>>(d_in, d_out, n, c.p.Q);
    c.launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "convert launch");
}

}  // namespace fheacc
