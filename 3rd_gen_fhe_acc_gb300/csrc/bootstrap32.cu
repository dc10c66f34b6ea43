// bootstrap32.cu -- stand-alone sub-steps of the 32-bit path (N = 1024,
// Q < 2^27): forward / inverse NTT of polynomial batches, one RLWE x RGSW
// product per CTA, and the extraction of NTT-domain RLWEs for the LWE key
// switch. They serve the parity entry points of the C ABI; the batched gate
// bootstrap itself runs in blind_rotate32.cu.
//
// Reference behaviour: NTT / iNTT (FHE_ACC_runtime/src/nbt.cpp:423-491),
// RLWE_mult_RGSW (RLWE.cpp:642-704), NTT_a_transpose + to_time_domain as used
// by LWE_keyswitch (RLWE.cpp:218-226, LWE.cpp:235-239).
#include "ctx.hpp"
#include "step32.cuh"
#include <algorithm>

namespace fheacc {
namespace dev {

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
                                                              size_t rgsw_stride,
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
        KeyU64Ref key{rgsw + ci * rgsw_stride};
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
        c.launches++;
    } else {
        cudaFuncSetAttribute(dev::ntt32_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        dev::ntt32_kernel<false><<<(unsigned)blocks, 256, smem, st>>>(d_polys, count, c.nc, c.d_fwd_tw,
                                                                      mu32_of(c.p.Q));
        c.launches++;
    }
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "ntt32 launch");
}

template <int DG>
static int launch_mult_rgsw_dg(Context &c, const uint64_t *d_acc, const uint64_t *d_rgsw, uint64_t *d_out,
                               size_t count, size_t stride, cudaStream_t st)
{
    const size_t smem = dev::step_smem_bytes<DG>();
    cudaFuncSetAttribute(dev::rlwe_mult_rgsw32_kernel<DG>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    size_t blocks = std::min<size_t>(count, (size_t)num_sms(c) * 4);
    dev::rlwe_mult_rgsw32_kernel<DG><<<(unsigned)blocks, 256, smem, st>>>(
        d_acc, d_rgsw, d_out, count, stride, c.nc, c.d_fwd_tw, c.d_inv_tw, c.p.BG_bits, c.dp.mu64);
    c.launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "rlwe_mult_rgsw32 launch");
}

int launch_rlwe_mult_rgsw32(Context &c, const uint64_t *d_acc, const uint64_t *d_rgsw, uint64_t *d_out,
                            size_t count, size_t stride, cudaStream_t st)
{
    if (!count) return FHEACC_OK;
    switch (c.p.digitG) {
    case 2: return launch_mult_rgsw_dg<2>(c, d_acc, d_rgsw, d_out, count, stride, st);
    case 3: return launch_mult_rgsw_dg<3>(c, d_acc, d_rgsw, d_out, count, stride, st);
    case 4: return launch_mult_rgsw_dg<4>(c, d_acc, d_rgsw, d_out, count, stride, st);
    default: return c.fail(FHEACC_EINVAL, "digitG must be 2..4 for the 32-bit path");
    }
}

int launch_extract_from_ntt32(Context &c, const uint64_t *d_rlwe, size_t count, uint32_t *d_extract,
                              cudaStream_t st)
{
    if (!count) return FHEACC_OK;
    size_t blocks = std::min<size_t>(count, (size_t)num_sms(c) * 16);
    dev::extract32_kernel<<<(unsigned)blocks, 64, 0, st>>>(d_rlwe, count, d_extract, c.nc, c.d_inv_tw);
    c.launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "extract32 launch");
}

}  // namespace fheacc
