// probe.cu -- measures the 32-bit IMAD throughput of the device, the
// denominator of the integer roofline reported for the blind-rotation kernel.
// Eight independent multiply-add chains per thread keep the pipe busy; the
// result of the chains is written only under a condition that never holds,
// so the work cannot be removed by the compiler and nothing is stored.
#include "ctx.hpp"

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

}  // namespace dev

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

}  // namespace fheacc
