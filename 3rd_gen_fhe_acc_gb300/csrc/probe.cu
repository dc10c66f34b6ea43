// probe.cu -- throughput probes behind the blind-rotation roofline.
//
// measure_imad_rate: the 32-bit IMAD throughput of the device, the denominator
// of the integer roofline. Eight independent multiply-add chains per thread
// keep the pipe busy; the result of the chains is written only under a
// condition that never holds, so the work cannot be removed by the compiler
// and nothing is stored.
//
// measure_l2_read_rate: the device's L2 read bandwidth, the peak the
// blind rotation's key streaming (RGSW words served from L2) is compared with.
//
// measure_components: the SM time of each piece of one RLWE x RGSW step when
// run alone at the blind-rotation kernel's occupancy (10-warp CTAs, two per
// SM): the forward, digit and inverse NTTs of ntt32.cuh on the context's
// twiddles, repeated in registers, and the multiply-accumulate (mac_chunk)
// streaming the context's bootstrap key from L2. Their sum per step is the
// time the pipeline would take with perfect overlap.
#include "ctx.hpp"
#include "step32.cuh"
#include <algorithm>

namespace fheacc {
namespace dev {

__global__ void imad_chain_kernel(uint32_t *sink, int iters, uint32_t a, uint32_t b)
{
    uint32_t x[8];
#pragma unroll
    for (int c = 0; c < 8; c++) x[c] = threadIdx.x + 17u * c;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < 8; c++) x[c] = x[c] * a + b;
    }
    uint32_t s = 0;
#pragma unroll
    for (int c = 0; c < 8; c++) s ^= x[c];
    if (s == 0x9E3779B9u && sink) sink[0] = s;
}

// Repeats one transform per warp `iters` times in registers (timing only;
// inputs are masked into the transform's input range every round).
template <int MODE>
__global__ void __launch_bounds__(320, 2) ntt_rate_kernel(uint32_t *sink, int iters, const __grid_constant__ Ntt32Consts c,
                                                          const uint2 *__restrict__ fwd_tw,
                                                          const uint2 *__restrict__ inv_tw, int bg_bits)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    uint32_t *bufs = reinterpret_cast<uint32_t *>(smem_raw);   // [10][1024]
    const int BG = 1 << bg_bits, cl = digit_table_copies_log2(bg_bits), BGC = BG << cl;
    uint32_t *t1 = bufs + 10 * kN32;
    uint2 *t23 = reinterpret_cast<uint2 *>(t1 + BGC), *t123 = t23 + BGC;
    for (int i = threadIdx.x; i < BGC; i += blockDim.x) {
        const uint64_t y = (uint64_t)(i >> cl);
        t1[i] = (uint32_t)(y * c.fw[1] % c.Q);
        t23[i] = make_uint2((uint32_t)(y * c.fw[2] % c.Q), (uint32_t)(y * c.fw[3] % c.Q));
        t123[i] = make_uint2(t1[i], t23[i].x);
    }
    __syncthreads();
    const DigitTables dt{t1, t23, t123, cl};
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t *buf = bufs + warp * kN32;
    uint32_t x[32];
#pragma unroll
    for (int r = 0; r < 32; r++) x[r] = (lane * 977u + r * 131u + blockIdx.x) % c.Q;
    for (int it = 0; it < iters; it++) {
        if (MODE == 0) {
#pragma unroll
            for (int r = 0; r < 32; r++) x[r] = min(x[r], x[r] - c.Q) & 0x3FFFFFFu;
            ntt_fwd_1024(x, c, fwd_tw, buf, lane);
        } else if (MODE == 1) {
#pragma unroll
            for (int r = 0; r < 32; r++) x[r] &= (uint32_t)BG - 1;
            ntt_fwd_1024_digit(x, c, fwd_tw, buf, dt, lane);
        } else {
#pragma unroll
            for (int r = 0; r < 32; r++) x[r] = min(x[r], x[r] - c.Q);
            ntt_inv_1024_noscale(x, c, inv_tw, buf, lane);
        }
    }
    uint32_t h = 0;
#pragma unroll
    for (int r = 0; r < 32; r++) h ^= x[r];
    if (h == 0x9E3779B9u && sink) sink[0] = h;
}

// Multiply-accumulate of one step per CTA and iteration with the digit
// warps' thread count, keys of the first steps of the bootstrap key (all
// residues) streamed from L2, results to a per-CTA accumulator.
template <int DG>
__global__ void __launch_bounds__(32 * (2 * DG + 2), 2) mac_rate_kernel(const uint32_t *__restrict__ btkey, int nkeys,
                                                                       uint32_t *accs, int iters, uint32_t Q,
                                                                       uint32_t qinv_neg)
{
    __shared__ __align__(16) uint32_t dbuf[2 * DG][kN32];
    for (int i = threadIdx.x; i < 2 * DG * kN32; i += blockDim.x) (&dbuf[0][0])[i] = (uint32_t)(i * 2654435761u) % (20 * Q);
    __syncthreads();
    uint4 *acc = reinterpret_cast<uint4 *>(accs + (size_t)blockIdx.x * 2048);
    const size_t rgsw_words = (size_t)DG * 4 * kN32;
    for (int it = 0; it < iters; it++) {
        const uint4 *key = reinterpret_cast<const uint4 *>(btkey + (size_t)((it * 7 + blockIdx.x) % nkeys) * rgsw_words);
        for (int u = threadIdx.x; u < 256; u += 32 * 2 * DG)
            if (threadIdx.x < 32 * 2 * DG) mac_chunk<DG>(u, key, dbuf, acc, Q, qinv_neg);
        __syncthreads();
    }
}

// Streaming read of a buffer that fits in L2 (after a warm-up pass it is
// L2-resident): every thread reads 16-byte words with ld.global.cg (cached in
// L2 only) over `passes` sweeps of its grid-strided share; the XOR of the
// words is stored only under a condition that never holds.
__global__ void l2_read_kernel(const uint4 *__restrict__ buf, size_t words, int passes, uint32_t *sink)
{
    uint32_t h = 0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (int p = 0; p < passes; p++) {
        for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += 4 * stride) {
            uint4 v[4];
#pragma unroll
            for (int u = 0; u < 4; u++) v[u] = i + u * stride < words ? __ldcg(buf + i + u * stride) : make_uint4(0, 0, 0, 0);
#pragma unroll
            for (int u = 0; u < 4; u++) h ^= v[u].x ^ v[u].y ^ v[u].z ^ v[u].w;
        }
    }
    if (h == 0x9E3779B9u && sink) sink[0] = h;
}

}  // namespace dev

template <class F>
static int time_best(Context &c, F launch, float *best_ms);

int measure_l2_read_rate(Context &c, double *bytes_per_s)
{
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device);
    int l2 = 0;
    cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, c.device);
    // a third of L2: resident after the first sweep on either L2 partition
    const size_t bytes = std::max<size_t>((size_t)std::max(l2, 1 << 20) / 3 / 4096 * 4096, 1 << 20);
    void *buf = nullptr;
    if (cudaMalloc(&buf, bytes) != cudaSuccess) {
        cudaGetLastError();
        return c.fail(FHEACC_ENOMEM, "L2 probe buffer");
    }
    cudaMemsetAsync(buf, 1, bytes, c.stream);
    const int blocks = (sms > 0 ? sms : 1) * 4, threads = 512, passes = 40;
    const size_t words = bytes / 16;
    float ms = 0;
    int rc = time_best(c, [&] {
        dev::l2_read_kernel<<<blocks, threads, 0, c.stream>>>((const uint4 *)buf, words, passes, nullptr);
    }, &ms);
    cudaFree(buf);
    if (rc) return rc;
    *bytes_per_s = (double)bytes * passes / (ms * 1e-3);
    return FHEACC_OK;
}

int measure_imad_rate(Context &c, double *imad_per_s)
{
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device);
    const int blocks = (sms > 0 ? sms : 1) * 8, threads = 256, iters = 20000;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 3; rep++) {
        cudaEventRecord(e0, c.stream);
        dev::imad_chain_kernel<<<blocks, threads, 0, c.stream>>>(nullptr, iters, 1664525u, 1013904223u);
        cudaEventRecord(e1, c.stream);
        cudaError_t e = cudaEventSynchronize(e1);
        if (e != cudaSuccess) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return c.cuda_fail(e, "imad probe");
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *imad_per_s = (double)blocks * threads * iters * 8 / (best * 1e-3);
    return FHEACC_OK;
}

// Best of two timed runs (after one warm-up) of `launch`, in ms.
template <class F>
static int time_best(Context &c, F launch, float *best_ms)
{
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    int rc = FHEACC_OK;
    for (int rep = 0; rep < 3 && !rc; rep++) {
        cudaEventRecord(e0, c.stream);
        launch();
        cudaEventRecord(e1, c.stream);
        cudaError_t e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e != cudaSuccess) {
            rc = c.cuda_fail(e, "component probe");
            break;
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *best_ms = best;
    return rc;
}

template <int DG>
static int time_mac(Context &c, uint32_t *accs, int blocks, int iters, float *ms)
{
    const int nkeys = std::min<int>(4 * (int)c.p.Br, (int)(c.p.n * c.p.digitR * c.p.Br));
    return time_best(c, [&] {
        dev::mac_rate_kernel<DG><<<blocks, 32 * (2 * DG + 2), 0, c.stream>>>(c.d_btkey, nkeys, accs, iters,
                                                                            (uint32_t)c.p.Q, c.dp.qinv_neg);
    }, ms);
}

int measure_components(Context &c, double ns[4])
{
    if (c.wide) return c.fail(FHEACC_EINVAL, "component probe: 32-bit parameter sets only");
    if (!c.d_btkey) return c.fail(FHEACC_ENOKEY, "component probe: bootstrap key not uploaded");
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device);
    if (sms < 1) sms = 1;
    const int blocks = 2 * sms, iters = 200;
    // the digit transform uses tables only for gadget bases up to 2^9 (as the
    // blind rotation does); above that it is the plain forward NTT
    const bool tables = c.p.BG_bits <= 9;
    const int bg = tables ? (int)c.p.BG_bits : 1;
    const size_t smem = 10 * dev::kN32 * sizeof(uint32_t) + ((20 * ((size_t)1 << bg)) << dev::digit_table_copies_log2(bg));
    float ms[4] = {0, 0, 0, 0};
    int rc = FHEACC_OK;
    auto k0 = dev::ntt_rate_kernel<0>, k1 = dev::ntt_rate_kernel<1>, k2 = dev::ntt_rate_kernel<2>;
    for (auto k : {k0, k1, k2})
        if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
            return c.cuda_fail(cudaGetLastError(), "component probe smem attribute");
    rc = time_best(c, [&] { k0<<<blocks, 320, smem, c.stream>>>(nullptr, iters, c.nc, c.d_fwd_tw, c.d_inv_tw, bg); }, &ms[0]);
    if (!rc && tables)
        rc = time_best(c, [&] { k1<<<blocks, 320, smem, c.stream>>>(nullptr, iters, c.nc, c.d_fwd_tw, c.d_inv_tw, bg); },
                       &ms[1]);
    else
        ms[1] = ms[0];
    if (!rc) rc = time_best(c, [&] { k2<<<blocks, 320, smem, c.stream>>>(nullptr, iters, c.nc, c.d_fwd_tw, c.d_inv_tw, bg); }, &ms[2]);
    if (rc) return rc;
    uint32_t *accs = nullptr;
    if (cudaMalloc(&accs, (size_t)blocks * 2048 * sizeof(uint32_t)) != cudaSuccess) {
        cudaGetLastError();
        return c.fail(FHEACC_ENOMEM, "component probe scratch");
    }
    const int mac_iters = 1000;
    switch (c.p.digitG) {
    case 2: rc = time_mac<2>(c, accs, blocks, mac_iters, &ms[3]); break;
    case 3: rc = time_mac<3>(c, accs, blocks, mac_iters, &ms[3]); break;
    case 4: rc = time_mac<4>(c, accs, blocks, mac_iters, &ms[3]); break;
    default: rc = c.fail(FHEACC_EINVAL, "component probe: digitG 2..4");
    }
    cudaFree(accs);
    if (rc) return rc;
    // SM time per unit: elapsed * SMs / units (10 warps x iters transforms per CTA)
    for (int i = 0; i < 3; i++) ns[i] = ms[i] * 1e6 * sms / ((double)blocks * 10 * iters);
    ns[3] = ms[3] * 1e6 * sms / ((double)blocks * mac_iters);
    return FHEACC_OK;
}

}  // namespace fheacc
