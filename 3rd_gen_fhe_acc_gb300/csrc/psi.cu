// psi.cu -- the RLWE-level operations of the reference's PSI application on
// the device: CMUX (RLWE.cpp:788-793), the RLWE blind rotation by an encrypted
// amount (blind_rotate, RLWE.cpp:824-838) and homo_expand (app.cpp:78-96),
// which turns digitG packed RLWEs into N RGSW ciphertexts. Their FPGA twins are
// the RLWE_MULT_RGSW / RLWESUBS instruction streams of fpga_homo_expand
// (myfpga.cpp:2278-2452); the reference's PSI test chains them
// (test.cpp:1510-1606): homo_expand, a CMUX tree selecting a database entry,
// then a blind rotation.
//
// Every operation is composed of the library's batched RLWE x RGSW kernels
// (bootstrap32.cu / bootstrap64.cu, which take one RGSW per item or one shared
// RGSW), expand_RLWE (expand.cu) and one elementwise kernel (RLWE subtraction,
// addition, and the NTT-domain rotation RLWE_rotate_freq, RLWE.cpp:411-430).
// Ciphertexts are canonical NTT-domain RLWEs, [count][2N] u64, as in the
// reference; results are bit-identical to it.
#include "ctx.hpp"
#include <algorithm>

namespace fheacc {
namespace dev {

enum { kEwSub = 0, kEwAdd = 1, kEwRot = 2 };

// out[i] = a[i] - b[i], a[i] + b[i], or a[i] * rot[e] (e = coefficient) mod Q
// for `count` RLWEs of 2N words; a and b step by a_stride / b_stride words per
// RLWE, out by 2N. Inputs canonical (< Q < 2^62).
__global__ void rlwe_elementwise_kernel(int mode, const uint64_t *__restrict__ a, size_t a_stride,
                                        const uint64_t *__restrict__ b, size_t b_stride,
                                        const uint64_t *__restrict__ rot, uint64_t *__restrict__ out,
                                        size_t count, int N, uint64_t Q)
{
    const size_t rw = 2 * (size_t)N, total = count * rw;
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        const size_t item = x / rw, w = x - item * rw;
        const uint64_t u = a[item * a_stride + w];
        uint64_t v;
        if (mode == kEwSub) {
            const uint64_t y = b[item * b_stride + w];
            v = u >= y ? u - y : u + Q - y;
        } else if (mode == kEwAdd) {
            const uint64_t s = u + b[item * b_stride + w];
            v = s >= Q ? s - Q : s;
        } else {
            v = (uint64_t)((unsigned __int128)u * rot[w & (size_t)(N - 1)] % Q);
        }
        out[x] = v;
    }
}

}  // namespace dev

static int launch_elementwise(Context &c, int mode, const uint64_t *a, size_t a_stride, const uint64_t *b,
                              size_t b_stride, const uint64_t *rot, uint64_t *out, size_t count, cudaStream_t st)
{
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device);
    const size_t words = count * 2 * (size_t)c.p.N;
    const size_t blocks = std::max<size_t>(1, std::min<size_t>((words + 255) / 256, (size_t)std::max(sms, 1) * 8));
    dev::rlwe_elementwise_kernel<<<(unsigned)blocks, 256, 0, st>>>(mode, a, a_stride, b, b_stride, rot, out, count,
                                                                  c.p.N, c.p.Q);
    c.launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "elementwise launch");
}

static int mult_rgsw(Context &c, const uint64_t *acc, const uint64_t *rgsw, size_t stride, uint64_t *out,
                     size_t count, cudaStream_t st)
{
    return c.wide ? launch_rlwe_mult_rgsw64(c, acc, rgsw, out, count, stride, st)
                  : launch_rlwe_mult_rgsw32(c, acc, rgsw, out, count, stride, st);
}

// CMUX of count pairs into `out` (contiguous): out = RLWE_mult_RGSW(c1 - c0, sel) + c0.
// scratch: 2 * count * 2N words. out may alias c0 when in_stride is 2N.
static int cmux_device(Context &c, const uint64_t *c0, const uint64_t *c1, size_t in_stride, const uint64_t *sel,
                       size_t sel_stride, uint64_t *out, size_t count, uint64_t *scratch, cudaStream_t st)
{
    const size_t rw = 2 * (size_t)c.p.N;
    uint64_t *diff = scratch, *mult = scratch + count * rw;
    int rc = launch_elementwise(c, dev::kEwSub, c1, in_stride, c0, in_stride, nullptr, diff, count, st);
    if (!rc) rc = mult_rgsw(c, diff, sel, sel_stride, mult, count, st);
    if (!rc) rc = launch_elementwise(c, dev::kEwAdd, mult, rw, c0, in_stride, nullptr, out, count, st);
    return rc;
}

}  // namespace fheacc

using namespace fheacc;

extern "C" {

int fheacc_cmux_async(fheacc_ctx *ctx, const uint64_t *d_c0, const uint64_t *d_c1, size_t in_stride,
                      const uint64_t *d_sel, int sel_shared, uint64_t *d_out, size_t count, void *stream)
{
    if (!ctx) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    const size_t rw = 2 * (size_t)c.p.N;
    if (count && (!d_c0 || !d_c1 || !d_sel || !d_out)) return c.fail(FHEACC_EINVAL, "null buffer");
    if (in_stride == 0) in_stride = rw;
    if (in_stride < rw) return c.fail(FHEACC_EINVAL, "CMUX input stride below one RLWE");
    if (!count) return FHEACC_OK;
    DeviceGuard g(c.device);
    cudaStream_t st = (cudaStream_t)stream;
    int rc = ensure_scratch(c, c.psi, 2 * count * rw * sizeof(uint64_t));
    if (rc) return rc;
    const size_t gw = (size_t)c.p.digitG * 4 * c.p.N;
    return cmux_device(c, d_c0, d_c1, in_stride, d_sel, sel_shared ? 0 : gw, d_out, count, (uint64_t *)c.psi.ptr,
                       st);
}

int fheacc_rlwe_blind_rotate_async(fheacc_ctx *ctx, const uint64_t *d_in, const uint64_t *d_rgsws, int forward,
                                   uint64_t *d_out, size_t count, void *stream)
{
    if (!ctx) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    if (count && (!d_in || !d_rgsws || !d_out)) return c.fail(FHEACC_EINVAL, "null buffer");
    if (!count) return FHEACC_OK;
    DeviceGuard g(c.device);
    cudaStream_t st = (cudaStream_t)stream;
    const int N = c.p.N, logN = c.wide ? 11 : 10;
    const size_t rw = 2 * (size_t)N, gw = (size_t)c.p.digitG * 4 * N;
    // tmp (rotated acc) + the CMUX scratch
    int rc = ensure_scratch(c, c.psi, 3 * count * rw * sizeof(uint64_t));
    if (rc) return rc;
    uint64_t *tmp = (uint64_t *)c.psi.ptr, *cm = tmp + count * rw;
    cudaError_t e = cudaMemcpyAsync(d_out, d_in, count * rw * sizeof(uint64_t), cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return c.cuda_fail(e, "blind rotate copy");
    const uint64_t *rot = forward ? c.d_rot_fwd : c.d_rot;
    for (int i = 0; i < logN && !rc; i++) {
        // tmp = RLWE_rotate_freq(acc, i, forward); acc = CMUX(acc, tmp, C[i])
        rc = launch_elementwise(c, dev::kEwRot, d_out, rw, nullptr, 0, rot + (size_t)i * N, tmp, count, st);
        if (!rc) rc = cmux_device(c, d_out, tmp, rw, d_rgsws + (size_t)i * gw, 0, d_out, count, cm, st);
    }
    return rc;
}

int fheacc_homo_expand(fheacc_ctx *ctx, const uint64_t *d_packed, const uint64_t *d_enc_sec, uint64_t *d_out,
                       void *stream)
{
    if (!ctx) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    if (!d_packed || !d_enc_sec || !d_out) return c.fail(FHEACC_EINVAL, "null buffer");
    DeviceGuard g(c.device);
    cudaStream_t st = (cudaStream_t)stream;
    const size_t N = (size_t)c.p.N, rw = 2 * N, dG = c.p.digitG, gw = dG * 4 * N;
    // all digits at once: the dG x N expanded RLWEs (the dG expansions level by
    // level, one launch per level) and their products with enc_sec (one launch)
    int rc = ensure_scratch(c, c.psi, 2 * dG * N * rw * sizeof(uint64_t));
    if (rc) return rc;
    uint64_t *u = (uint64_t *)c.psi.ptr, *m = u + dG * N * rw;
    rc = expand_device(c, d_packed, u, st, dG);
    if (!rc) rc = mult_rgsw(c, u, d_enc_sec, 0, m, dG * N, st);
    for (size_t j = 0; j < dG && !rc; j++) {
        // RGSW i, row j: c_text[j][0] = m[j][i], c_text[j][1] = u[j][i]
        cudaError_t e = cudaMemcpy2DAsync(d_out + (j * 2 + 0) * rw, gw * sizeof(uint64_t), m + j * N * rw,
                                          rw * sizeof(uint64_t), rw * sizeof(uint64_t), N, cudaMemcpyDeviceToDevice,
                                          st);
        if (e == cudaSuccess)
            e = cudaMemcpy2DAsync(d_out + (j * 2 + 1) * rw, gw * sizeof(uint64_t), u + j * N * rw,
                                  rw * sizeof(uint64_t), rw * sizeof(uint64_t), N, cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) rc = c.cuda_fail(e, "homo_expand rows");
    }
    return rc;
}

}  // extern "C"
