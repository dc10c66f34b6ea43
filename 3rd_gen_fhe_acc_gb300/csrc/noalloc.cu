// noalloc.cu -- gate bootstrapping without any device allocation.
//
// fheacc_bootstrap_async grows the context's scratch (blind-rotation
// accumulators and extracted RLWEs) with cudaMalloc / cudaFree when a batch is
// larger than any before it. Some callers cannot let that happen on their hot
// path: cudaFree synchronises the whole device (stalling unrelated streams of a
// serving process), a process may run under a fixed device-memory reservation
// with nothing left to grow into, and a real-time loop may forbid allocator
// calls outright. fheacc_bootstrap_noalloc serves them: its scratch is the
// file-scope device array below, reserved when the library is loaded, so a
// call allocates nothing. The caller still provides inputs and outputs.
#include "ctx.hpp"
#include <mutex>

namespace fheacc {

// Scratch of fheacc_bootstrap_noalloc for at most FHEACC_NOALLOC_MAX_GATES
// gates: blind-rotation accumulators (2048 words per gate) followed by the
// extracted RLWEs (kExtractStride words per gate). 776 KiB, held on every GPU
// that loads the library until the process exits.
constexpr size_t kNoAllocAccWords = (size_t)FHEACC_NOALLOC_MAX_GATES * 2048 + kClaimWords;
constexpr size_t kNoAllocWords = kNoAllocAccWords + (size_t)FHEACC_NOALLOC_MAX_GATES * kExtractStride;
static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoAllocWords];

// The split key switch of a call (launch_lwe_keyswitch32 with partial sums)
// keeps ks_row 64-bit sums per gate in the accumulator area, 2048 words per
// gate; ks_row is at most 4 * kKsMaxThreads words (the key-switch CTA width),
// and the upload refuses wider rows, so the sums fit.
static_assert(4 * kKsMaxThreads * sizeof(uint64_t) <= 2048 * sizeof(uint32_t),
              "key-switch partial sums must fit in one gate's accumulator words");

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
uint32_t *g_noalloc_ptr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device. In host code the
// array's name is only a stand-in for the symbol, so the address is looked up
// once per device (with that device current) and cached.
int noalloc_scratch(Context &c, uint32_t **out)
{
    if (c.device < 0 || c.device >= kMaxDevices) return c.fail(FHEACC_EINVAL, "device index out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[c.device]) {
        void *ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) {
            cudaGetLastError();
            return c.cuda_fail(e != cudaSuccess ? e : cudaErrorInvalidSymbol, "no-alloc scratch address");
        }
        g_noalloc_ptr[c.device] = static_cast<uint32_t *>(ptr);
    }
    *out = g_noalloc_ptr[c.device];
    return FHEACC_OK;
}
}  // namespace

}  // namespace fheacc

using namespace fheacc;

extern "C" int fheacc_bootstrap_noalloc(fheacc_ctx *ctx, const uint64_t *d_c1, const uint64_t *d_c2,
                                        const int32_t *d_gates, size_t count, uint64_t *d_out, uint32_t flags,
                                        void *stream)
{
    if (!ctx) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    if (count > FHEACC_NOALLOC_MAX_GATES)
        return c.fail(FHEACC_EINVAL, "fheacc_bootstrap_noalloc: count exceeds FHEACC_NOALLOC_MAX_GATES (64); split the "
                                     "batch or use fheacc_bootstrap_async");
    if (c.p.N != 1024) return c.fail(FHEACC_EINVAL, "fheacc_bootstrap_noalloc: scratch is sized for N = 1024");
    if (count == 0) return FHEACC_OK;
    if (!d_c1 || !d_c2 || !d_gates || !d_out) return c.fail(FHEACC_EINVAL, "null buffer");
    if (!c.d_btkey) return c.fail(FHEACC_ENOKEY, "bootstrap key not uploaded");
    if (!c.d_kskey) return c.fail(FHEACC_ENOKEY, "LWE key-switch key not uploaded");
    if (c.dp.ks_row > 4 * kKsMaxThreads) return c.fail(FHEACC_EINVAL, "fheacc_bootstrap_noalloc: n too large");
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != c.device) cudaSetDevice(c.device);
    uint32_t *scratch = nullptr;
    int rc = noalloc_scratch(c, &scratch);
    // The array keeps the previous call's words. The accumulators and the
    // extracted RLWEs are written by this call before they are read (the blind
    // rotation's prologue and epilogue); the two parts that must start at zero
    // are reset on the stream with cudaMemsetAsync, which allocates nothing:
    // the blind rotation's claim counter (after the accumulators) and the
    // split key switch's 64-bit partial sums (in the accumulator area, free
    // once the blind rotation is done).
    if (rc == FHEACC_OK) {
        cudaStream_t st = (cudaStream_t)stream;
        uint32_t *accs = scratch, *ext = scratch + kNoAllocAccWords;
        const bool prof = (flags & FHEACC_FLAG_PROFILE) != 0;
        flags &= ~(uint32_t)FHEACC_FLAG_PROFILE;
        if (prof) cudaEventRecord(c.prof[0], st);
        rc = launch_blind_rotate32_with(c, d_c1, d_c2, d_gates, count, flags, accs, ext, st);
        if (rc == FHEACC_OK && prof) cudaEventRecord(c.prof[1], st);
        if (rc == FHEACC_OK)
            rc = launch_lwe_keyswitch32(c, ext, count, true, d_out, st, accs,
                                        (size_t)FHEACC_NOALLOC_MAX_GATES * 2048 * sizeof(uint32_t));
        if (rc == FHEACC_OK && prof) cudaEventRecord(c.prof[2], st);
        if (rc == FHEACC_OK) {
            cudaError_t e = cudaEventRecord(c.done, st);
            if (e != cudaSuccess) rc = c.cuda_fail(e, "event record");
        }
    }
    if (prev >= 0 && prev != c.device) cudaSetDevice(prev);
    return rc;
}
