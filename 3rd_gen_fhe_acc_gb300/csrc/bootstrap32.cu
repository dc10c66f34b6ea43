// bootstrap32.cu -- blind rotation of FHEW/AP gate bootstrapping for N = 1024
// and Q < 2^27 (32-bit words), plus the NTT and RLWE x RGSW sub-steps.
//
// Reference behaviour: RLWE::eval_bootstrap (FHE_ACC_runtime/src/RLWE.cpp:726-767)
// with RLWE_mult_RGSW (RLWE.cpp:642-704), digit_decompose (RLWE.cpp:623-640) and
// acc_initialization (RLWE.cpp:706-724); the FPGA cores this replaces are
// iNTT_module.sv, NTT_leading_stage.sv/NTT_stage.sv, poly_mult_RLWE.sv and
// accumulator.sv.
//
// One CTA works on one ciphertext at a time and keeps its accumulator in shared
// memory for the whole blind rotation; the grid is persistent (one wave of
// CTAs loops over the batch). All CTAs start together and each step costs the
// same, so the CTAs move through the bootstrapping key in near lockstep and the
// 23 RGSW keys of a step are read from HBM about once per wave and then served
// from L2. Each RLWE x RGSW step is three phases separated by __syncthreads:
//   1. warps 0, 1: inverse NTT of acc.a, acc.b  -> canonical time domain
//   2. warp (p, h): digit h of poly p, forward NTT (2 * digitG warps)
//   3. all threads: acc'[P][k] = sum_{p,h} D[p][h][k] * K[h][p][P][k] mod Q,
//      64-bit accumulation, one Barrett reduction per output, keys streamed
//      from L2/HBM with 128-bit loads.
#include "ctx.hpp"
#include <algorithm>

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

// ------------------------------------------------------------------ kernels

// Forward / inverse NTT of `count` u64 polys in place, one warp per poly.
template <bool INV>
__global__ void __launch_bounds__(256) ntt32_kernel(uint64_t *polys, size_t count, const __grid_constant__ Ntt32Consts c,
                                                    const uint2 *__restrict__ tw, uint32_t mu32)
{
    extern __shared__ uint32_t smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t *buf = smem + warp * kPadN;
    for (size_t pi = (size_t)blockIdx.x * 8 + warp; pi < count; pi += (size_t)gridDim.x * 8) {
        uint64_t *poly = polys + pi * 1024;
        uint32_t x[32];
        if (!INV) {
#pragma unroll
            for (int r = 0; r < 32; r++) x[r] = (uint32_t)poly[lane + 32 * r];
            ntt_fwd_1024(x, c, tw, buf, lane);
#pragma unroll
            for (int r = 0; r < 32; r++) buf[33 * lane + r] = reduce32(x[r], mu32, c.Q);
            __syncwarp();
#pragma unroll
            for (int r = 0; r < 32; r++) poly[lane + 32 * r] = buf[pad32(lane + 32 * r)];
            __syncwarp();
        } else {
#pragma unroll
            for (int r = 0; r < 32; r++) buf[pad32(lane + 32 * r)] = (uint32_t)poly[lane + 32 * r];
            __syncwarp();
#pragma unroll
            for (int r = 0; r < 32; r++) x[r] = buf[33 * lane + r];
            ntt_inv_1024(x, c, tw, buf, lane);
#pragma unroll
            for (int r = 0; r < 32; r++) poly[lane + 32 * r] = x[r];
            __syncwarp();
        }
    }
}

// RLWE_mult_RGSW of count (acc, RGSW) pairs in the reference's u64 layouts.
template <int DG>
__global__ void __launch_bounds__(256) rlwe_mult_rgsw32_kernel(const uint64_t *__restrict__ acc_in,
                                                              const uint64_t *__restrict__ rgsw,
                                                              uint64_t *__restrict__ acc_out, size_t count,
                                                              const __grid_constant__ Ntt32Consts c,
                                                              const uint2 *__restrict__ fwd_tw,
                                                              const uint2 *__restrict__ inv_tw, uint32_t bg_bits,
                                                              uint64_t mu64)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    StepSmem<DG> &s = *reinterpret_cast<StepSmem<DG> *>(smem_raw);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (size_t ci = blockIdx.x; ci < count; ci += gridDim.x) {
        const uint64_t *in = acc_in + ci * 2048;
        for (int e = threadIdx.x; e < 2048; e += blockDim.x) {
            const int P = e >> 10, k = e & 1023;
            s.acc[P][pad32(k)] = (uint32_t)in[e];
        }
        __syncthreads();
        KeyU64Ref key{rgsw + ci * (size_t)DG * 4 * 1024};
        rlwe_x_rgsw_step<DG>(s, c, fwd_tw, inv_tw, key, bg_bits, mu64, warp, lane);
        uint64_t *out = acc_out + ci * 2048;
        for (int e = threadIdx.x; e < 2048; e += blockDim.x) {
            const int P = e >> 10, k = e & 1023;
            const uint32_t v = s.acc[P][pad32(k)];
            out[e] = v >= c.Q ? v - c.Q : v;
        }
        __syncthreads();
    }
}

struct BrArgs {
    const uint64_t *c1, *c2;
    const int32_t *gates;
    size_t count;
    const uint32_t *btkey;
    uint64_t *acc_out;      // optional: NTT accumulators [count][2N] (canonical)
    uint32_t *extract;      // optional: [count][kExtractStride] time-domain a (transposed), b0
    int n;
    uint32_t q, embed, Br, digitR, bg_bits, flags;
    uint64_t mu64;
    uint64_t gate_constant[8];
};

// Batched blind rotation: LWE_evaluate, acc_initialization, the n*digitR
// RLWE x RGSW steps (residue 0 skipped unless FPGA-compatible), then either the
// NTT accumulator or the extracted time-domain RLWE is written out.
template <int DG>
__global__ void __launch_bounds__(256) blind_rotate32_kernel(const __grid_constant__ BrArgs A,
                                                            const __grid_constant__ Ntt32Consts c,
                                                            const uint2 *__restrict__ fwd_tw,
                                                            const uint2 *__restrict__ inv_tw, uint32_t mu32)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    StepSmem<DG> &s = *reinterpret_cast<StepSmem<DG> *>(smem_raw);
    uint16_t *lwe_a = reinterpret_cast<uint16_t *>(smem_raw + sizeof(StepSmem<DG>));
    __shared__ uint32_t lwe_b, qb1, qb2;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n = A.n;
    const uint32_t q = A.q, qmask = q - 1;
    const size_t rgsw_words = (size_t)DG * 4 * 1024;

    for (size_t ci = blockIdx.x; ci < A.count; ci += gridDim.x) {
        // LWE_evaluate (LWE.cpp:203-222); q is a power of two
        int g = A.gates[ci];
        const bool x2 = (g == 4 || g == 5);
        const uint64_t *c1 = A.c1 + ci * (size_t)(n + 1), *c2 = A.c2 + ci * (size_t)(n + 1);
        for (int i = threadIdx.x; i <= n; i += blockDim.x) {
            uint64_t v = x2 ? 2 * (c1[i] - c2[i]) : c1[i] + c2[i];
            v &= qmask;
            if (i < n) lwe_a[i] = (uint16_t)v;
            else lwe_b = (uint32_t)v;
        }
        if (threadIdx.x == 0) {
            const uint64_t gc = A.gate_constant[(unsigned)g < 6u ? g : 6];
            qb1 = (uint32_t)(gc & qmask);
            qb2 = (qb1 + q / 2) & qmask;
        }
        __syncthreads();
        // acc_initialization (RLWE.cpp:706-724): a = 0, b = test vector, NTT
        if (warp == 0) {
            const uint32_t Q8 = (uint32_t)(c.Q / 8 + 1), negQ8 = c.Q - Q8;
            const uint32_t b1 = qb1, b2 = qb2, val = lwe_b;
            uint32_t x[32];
#pragma unroll
            for (int r = 0; r < 32; r++) {
                const uint32_t idx = lane + 32 * r;
                uint32_t v = 0;
                if (idx % A.embed == 0 && idx / A.embed < q / 2) {
                    const uint32_t tmp = (val - idx / A.embed) & qmask;
                    if (b1 < b2) v = (tmp >= b1 && tmp < b2) ? negQ8 : Q8;
                    else v = (tmp >= b2 && tmp < b1) ? Q8 : negQ8;
                }
                x[r] = v;
            }
            ntt_fwd_1024(x, c, fwd_tw, s.dbuf[0], lane);
#pragma unroll
            for (int r = 0; r < 32; r++) s.acc[1][33 * lane + r] = reduce32(x[r], mu32, c.Q);
        } else {
            for (int e = threadIdx.x - 32; e < kPadN; e += blockDim.x - 32) s.acc[0][e] = 0;
        }
        __syncthreads();
        // blind rotation (RLWE.cpp:754-767)
        for (int i = 0; i < n; i++) {
            uint32_t nega = (q - lwe_a[i]) & qmask;
            for (uint32_t j = 0; j < A.digitR; j++) {
                const uint32_t r = nega % A.Br;
                nega /= A.Br;
                if (r == 0 && !(A.flags & FHEACC_FLAG_FPGA_COMPAT)) continue;
                const size_t blk = ((size_t)(i * A.digitR + j) * A.Br + r) * rgsw_words;
                KeyU32 key{A.btkey + blk};
                rlwe_x_rgsw_step<DG>(s, c, fwd_tw, inv_tw, key, A.bg_bits, A.mu64, warp, lane);
            }
        }
        // output
        if (A.extract) {
            phase_intt<DG>(s, c, inv_tw, warp, lane, true);
            __syncthreads();
            uint32_t *ext = A.extract + ci * kExtractStride;
            for (int e = threadIdx.x; e < 1024; e += blockDim.x) ext[e] = s.tbuf[0][pad32(e)];
            if (threadIdx.x == 0) ext[1024] = s.tbuf[1][0];
        } else {
            uint64_t *out = A.acc_out + ci * 2048;
            for (int e = threadIdx.x; e < 2048; e += blockDim.x) {
                const uint32_t v = s.acc[e >> 10][pad32(e & 1023)];
                out[e] = v >= c.Q ? v - c.Q : v;
            }
        }
        __syncthreads();
    }
}

// Extraction of NTT RLWEs given in u64: NTT_a_transpose, inverse NTT of both
// polys, a[N] and b[0] to the extract layout (LWE.cpp:235-239).
__global__ void __launch_bounds__(64) extract32_kernel(const uint64_t *__restrict__ rlwe, size_t count,
                                                      uint32_t *__restrict__ extract,
                                                      const __grid_constant__ Ntt32Consts c,
                                                      const uint2 *__restrict__ inv_tw)
{
    __shared__ uint32_t buf[2][kPadN];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (size_t ci = blockIdx.x; ci < count; ci += gridDim.x) {
        const uint64_t *in = rlwe + ci * 2048 + warp * 1024;
        uint32_t x[32];
#pragma unroll
        for (int r = 0; r < 32; r++) {
            const int e = 32 * lane + r;
            x[r] = (uint32_t)in[warp == 0 ? 1023 - e : e];
        }
        ntt_inv_1024(x, c, inv_tw, buf[warp], lane);
        uint32_t *ext = extract + ci * kExtractStride;
        if (warp == 0) {
#pragma unroll
            for (int r = 0; r < 32; r++) ext[lane + 32 * r] = x[r];
        } else if (lane == 0) {
            ext[1024] = x[0];
        }
        __syncthreads();
    }
}

template <int DG>
static size_t step_smem_bytes()
{
    return sizeof(StepSmem<DG>);
}

}  // namespace dev

static uint32_t mu32_of(uint64_t Q) { return (uint32_t)((1ULL << 32) / Q); }

static int num_sms(Context &c)
{
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, c.device);
    return v > 0 ? v : 1;
}

int launch_ntt32(Context &c, uint64_t *d_polys, size_t count, bool inverse, cudaStream_t st)
{
    if (!count) return FHEACC_OK;
    const size_t smem = 8 * dev::kPadN * sizeof(uint32_t);
    size_t blocks = std::min<size_t>((count + 7) / 8, (size_t)num_sms(c) * 8);
    if (inverse) {
        cudaFuncSetAttribute(dev::ntt32_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        dev::ntt32_kernel<true><<<(unsigned)blocks, 256, smem, st>>>(d_polys, count, c.nc, c.d_inv_tw,
                                                                     mu32_of(c.p.Q));
    } else {
        cudaFuncSetAttribute(dev::ntt32_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        dev::ntt32_kernel<false><<<(unsigned)blocks, 256, smem, st>>>(d_polys, count, c.nc, c.d_fwd_tw,
                                                                      mu32_of(c.p.Q));
    }
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "ntt32 launch");
}

template <int DG>
static int launch_mult_rgsw_dg(Context &c, const uint64_t *d_acc, const uint64_t *d_rgsw, uint64_t *d_out,
                               size_t count, cudaStream_t st)
{
    const size_t smem = dev::step_smem_bytes<DG>();
    cudaFuncSetAttribute(dev::rlwe_mult_rgsw32_kernel<DG>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    size_t blocks = std::min<size_t>(count, (size_t)num_sms(c) * 4);
    dev::rlwe_mult_rgsw32_kernel<DG><<<(unsigned)blocks, 256, smem, st>>>(
        d_acc, d_rgsw, d_out, count, c.nc, c.d_fwd_tw, c.d_inv_tw, c.p.BG_bits, c.dp.mu64);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "rlwe_mult_rgsw32 launch");
}

int launch_rlwe_mult_rgsw32(Context &c, const uint64_t *d_acc, const uint64_t *d_rgsw, uint64_t *d_out,
                            size_t count, cudaStream_t st)
{
    if (!count) return FHEACC_OK;
    switch (c.p.digitG) {
    case 2: return launch_mult_rgsw_dg<2>(c, d_acc, d_rgsw, d_out, count, st);
    case 3: return launch_mult_rgsw_dg<3>(c, d_acc, d_rgsw, d_out, count, st);
    case 4: return launch_mult_rgsw_dg<4>(c, d_acc, d_rgsw, d_out, count, st);
    default: return c.fail(FHEACC_EINVAL, "digitG must be 2..4 for the 32-bit path");
    }
}

template <int DG>
static int launch_br_dg(Context &c, const dev::BrArgs &A, int max_ctas, cudaStream_t st)
{
    const size_t smem = dev::step_smem_bytes<DG>() + ((size_t)c.p.n * 2 + 15) / 16 * 16;
    cudaError_t e = cudaFuncSetAttribute(dev::blind_rotate32_kernel<DG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return c.cuda_fail(e, "blind_rotate32 smem attribute");
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dev::blind_rotate32_kernel<DG>, 256, smem);
    if (per_sm < 1) per_sm = 1;
    size_t blocks = std::min<size_t>(A.count, (size_t)num_sms(c) * per_sm);
    if (max_ctas > 0) blocks = std::min<size_t>(blocks, (size_t)max_ctas);
    dev::blind_rotate32_kernel<DG><<<(unsigned)blocks, 256, smem, st>>>(A, c.nc, c.d_fwd_tw, c.d_inv_tw,
                                                                        mu32_of(c.p.Q));
    e = cudaGetLastError();
    return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "blind_rotate32 launch");
}

int launch_blind_rotate32(Context &c, const uint64_t *d_c1, const uint64_t *d_c2, const int32_t *d_gates,
                          size_t count, uint32_t flags, uint64_t *d_acc_out, uint32_t *d_extract, int max_ctas,
                          cudaStream_t st)
{
    if (!count) return FHEACC_OK;
    if (!c.d_btkey) return c.fail(FHEACC_ENOKEY, "bootstrap key not uploaded");
    dev::BrArgs A{};
    A.c1 = d_c1; A.c2 = d_c2; A.gates = d_gates; A.count = count;
    A.btkey = c.d_btkey; A.acc_out = d_acc_out; A.extract = d_extract;
    A.n = c.p.n; A.q = c.p.q; A.embed = c.dp.embed; A.Br = c.p.Br; A.digitR = c.p.digitR;
    A.bg_bits = c.p.BG_bits; A.flags = flags; A.mu64 = c.dp.mu64;
    for (int i = 0; i < 8; i++) A.gate_constant[i] = c.dp.gate_constant[i];
    switch (c.p.digitG) {
    case 2: return launch_br_dg<2>(c, A, max_ctas, st);
    case 3: return launch_br_dg<3>(c, A, max_ctas, st);
    case 4: return launch_br_dg<4>(c, A, max_ctas, st);
    default: return c.fail(FHEACC_EINVAL, "digitG must be 2..4 for the 32-bit path");
    }
}

int launch_extract_from_ntt32(Context &c, const uint64_t *d_rlwe, size_t count, uint32_t *d_extract,
                              cudaStream_t st)
{
    if (!count) return FHEACC_OK;
    size_t blocks = std::min<size_t>(count, (size_t)num_sms(c) * 16);
    dev::extract32_kernel<<<(unsigned)blocks, 64, 0, st>>>(d_rlwe, count, d_extract, c.nc, c.d_inv_tw);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "extract32 launch");
}

}  // namespace fheacc
