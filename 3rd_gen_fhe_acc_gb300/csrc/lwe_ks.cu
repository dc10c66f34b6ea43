// lwe_ks.cu -- RLWE -> LWE key switch and modulus switch, 32-bit words.
//
// Reference behaviour: LWE::LWE_keyswitch (FHE_ACC_runtime/src/LWE.cpp:233-253)
// and LWE::LWE_modswitch / scale_round (LWE.cpp:255-269). The reference's FPGA
// path runs these on the host (myfpga.cpp:1519-1523); here they run on the GPU
// right after the blind rotation.
//
// Input is the extracted RLWE (time-domain a[N] after NTT_a_transpose, and
// b[0]). For every coefficient i < N and digit j < digitKS the LWE row
// kskey[d][j][i], d = base-Bks digit j of a[i], is subtracted. One CTA per
// ciphertext: the digits are computed once into shared memory, then the CTA
// walks the N * digitKS rows; a row is n+1 consecutive words, read by
// consecutive threads (coalesced). Sums are kept in 64-bit registers without
// reduction (N * digitKS * Q < 2^64) and reduced once at the end; the modulus
// switch is fused into the same epilogue.
#include "ctx.hpp"
#include <algorithm>

namespace fheacc {
namespace dev {

struct KsArgs {
    const uint32_t *ext;
    size_t count;
    const uint32_t *kskey;
    uint64_t *out;
    const uint32_t *out_idx;   // optional: ciphertext ci is written to out + out_idx[ci] * (n+1)
    int n, N, digitKS;
    uint32_t Bks, ks_row, q, modswitch;
    uint64_t Q;
};

__device__ __forceinline__ uint64_t scale_round_dev(uint64_t x, uint64_t new_mod, uint64_t old_mod)
{
    // LWE.cpp:255-260: (old + 2 x new) / (2 old), exact integer
    unsigned __int128 num = (unsigned __int128)old_mod + 2 * (unsigned __int128)x * new_mod;
    return (uint64_t)(num / (2 * (unsigned __int128)old_mod));
}

// One CTA per ciphertext, one thread per four words of a key row (ks_row / 4
// threads, one 128-bit load per row). The CTA puts the ciphertext's base-Bks
// digits in shared memory, then walks the N * digitKS rows it selects
// (kskey[d][j][i]), kKsUnroll rows per iteration so that each thread has that
// many independent loads in flight, with 64-bit sums.
constexpr int kKsUnroll = 8;

__global__ void __launch_bounds__(kKsMaxThreads) lwe_ks32_kernel(const __grid_constant__ KsArgs A)
{
    extern __shared__ uint8_t digits[];   // [N][digitKS]
    const int n = A.n, N = A.N, D = A.digitKS, t = threadIdx.x;
    const uint32_t Q = (uint32_t)A.Q;
    const size_t rs4 = A.ks_row / 4;
    const uint4 *key4 = reinterpret_cast<const uint4 *>(A.kskey);
    for (size_t ci = blockIdx.x; ci < A.count; ci += gridDim.x) {
        const uint32_t *ext = A.ext + ci * kExtractStride;
        for (int i = t; i < N; i += blockDim.x) {
            uint32_t a = ext[i];
            for (int j = 0; j < D; j++) {
                digits[i * D + j] = (uint8_t)(a % A.Bks);
                a /= A.Bks;
            }
        }
        __syncthreads();
        uint64_t s0 = 0, s1 = 0, s2 = 0, s3 = 0;
        const int total = N * D;
        int i = 0, j = 0;   // (coefficient, digit) of row r0 + u
        for (int r0 = 0; r0 < total; r0 += kKsUnroll) {
            uint4 v[kKsUnroll];
#pragma unroll
            for (int u = 0; u < kKsUnroll; u++) {
                v[u] = make_uint4(0, 0, 0, 0);
                if (r0 + u < total) {
                    const uint32_t d = digits[r0 + u];
                    v[u] = __ldg(key4 + ((size_t)(d * D + j) * N + i) * rs4 + t);
                }
                if (++j == D) {
                    j = 0;
                    ++i;
                }
            }
#pragma unroll
            for (int u = 0; u < kKsUnroll; u++) {
                s0 += v[u].x;
                s1 += v[u].y;
                s2 += v[u].z;
                s3 += v[u].w;
            }
        }
        const uint32_t b0 = ext[N];
        const uint32_t Q8 = Q / 8 + 1;
        uint64_t *out = A.out + (A.out_idx ? (size_t)A.out_idx[ci] : ci) * (size_t)(n + 1);
        const uint64_t sums[4] = {s0, s1, s2, s3};
#pragma unroll
        for (int c = 0; c < 4; c++) {
            const int k = 4 * t + c;
            if (k <= n) {
                const uint64_t s = sums[c] % Q;
                uint64_t v;
                if (k < n) v = s ? Q - s : 0;
                else v = ((uint64_t)(b0 + Q8) % Q + Q - s) % Q;
                out[k] = A.modswitch ? scale_round_dev(v, A.q, A.Q) : v;
            }
        }
        __syncthreads();
    }
}

// Split form for a few ciphertexts (the one-gate launches): CTA (ci, slice)
// sums rows [slice * rows_per, ...) of ciphertext ci and adds its 64-bit
// partial sums into part[ci][ks_row] (zeroed before; the sums stay below
// N * digitKS * Q < 2^64); ks_final_kernel reduces them.
__global__ void __launch_bounds__(kKsMaxThreads) ks_partial_kernel(const __grid_constant__ KsArgs A,
                                                                   unsigned long long *part, int slices)
{
    const int N = A.N, D = A.digitKS, t = threadIdx.x;
    const size_t rs4 = A.ks_row / 4;
    const uint4 *key4 = reinterpret_cast<const uint4 *>(A.kskey);
    const int total = N * D, per = (total + slices - 1) / slices;
    const size_t ci = blockIdx.x / slices;
    const int r0 = (int)(blockIdx.x % slices) * per, r1 = min(total, r0 + per);
    if (ci >= A.count) return;
    const uint32_t *ext = A.ext + ci * kExtractStride;
    uint64_t s0 = 0, s1 = 0, s2 = 0, s3 = 0;
    for (int r = r0; r < r1; r++) {
        const int i = r / D, j = r - i * D;
        uint32_t a = ext[i];
        for (int jj = 0; jj < j; jj++) a /= A.Bks;
        const uint32_t d = a % A.Bks;
        const uint4 v = __ldg(key4 + ((size_t)(d * D + j) * N + i) * rs4 + t);
        s0 += v.x;
        s1 += v.y;
        s2 += v.z;
        s3 += v.w;
    }
    unsigned long long *p = part + ci * A.ks_row + 4 * (size_t)t;
    atomicAdd(p + 0, (unsigned long long)s0);
    atomicAdd(p + 1, (unsigned long long)s1);
    atomicAdd(p + 2, (unsigned long long)s2);
    atomicAdd(p + 3, (unsigned long long)s3);
}

__global__ void ks_final_kernel(const __grid_constant__ KsArgs A, const unsigned long long *part)
{
    const uint32_t Q = (uint32_t)A.Q, Q8 = Q / 8 + 1;
    const size_t w = (size_t)A.n + 1;
    for (size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x; x < A.count * w; x += (size_t)gridDim.x * blockDim.x) {
        const size_t ci = x / w;
        const int k = (int)(x - ci * w);
        const uint64_t sm = part[ci * A.ks_row + k] % Q;
        uint64_t v;
        if (k < A.n) v = sm ? Q - sm : 0;
        else v = ((uint64_t)(A.ext[ci * kExtractStride + A.N] + Q8) % Q + Q - sm) % Q;
        A.out[x] = A.modswitch ? scale_round_dev(v, A.q, A.Q) : v;
    }
}

__global__ void modswitch_kernel(const uint64_t *__restrict__ in, uint64_t *__restrict__ out, size_t words,
                                 uint64_t q, uint64_t Q)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += (size_t)gridDim.x * blockDim.x)
        out[i] = scale_round_dev(in[i], q, Q);
}

}  // namespace dev

int launch_lwe_keyswitch32(Context &c, const uint32_t *d_extract, size_t count, bool modswitch, uint64_t *d_out,
                           cudaStream_t st, uint64_t *d_partials)
{
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device);
    // a few ciphertexts: split each one's rows over many CTAs
    if (!d_partials || count == 0 || count >= 2 * (size_t)std::max(sms, 1) || !c.d_kskey ||
        c.p.n + 1 > 4 * kKsMaxThreads)
        return launch_lwe_keyswitch32_indexed(c, d_extract, count, modswitch, d_out, nullptr, st);
    dev::KsArgs A{};
    A.ext = d_extract; A.count = count; A.kskey = c.d_kskey; A.out = d_out; A.out_idx = nullptr;
    A.n = c.p.n; A.N = c.p.N; A.digitKS = (int)c.p.digitKS; A.Bks = c.p.Bks; A.ks_row = c.dp.ks_row;
    A.q = c.p.q; A.modswitch = modswitch ? 1u : 0u; A.Q = c.p.Q;
    const int rows = c.p.N * (int)c.p.digitKS;
    // about 8 CTAs per SM, at least 48 rows each
    const int slices = (int)std::max<size_t>(1, std::min<size_t>((size_t)rows / 48, (size_t)sms * 8 / count));
    cudaError_t e = cudaMemsetAsync(d_partials, 0, count * c.dp.ks_row * sizeof(uint64_t), st);
    if (e != cudaSuccess) return c.cuda_fail(e, "key switch partials reset");
    dev::ks_partial_kernel<<<(unsigned)(count * slices), c.dp.ks_row / 4, 0, st>>>(
        A, reinterpret_cast<unsigned long long *>(d_partials), slices);
    c.launches++;
    e = cudaGetLastError();
    if (e != cudaSuccess) return c.cuda_fail(e, "key switch partial launch");
    const size_t words = count * ((size_t)c.p.n + 1);
    dev::ks_final_kernel<<<(unsigned)std::min<size_t>((words + 255) / 256, 1024), 256, 0, st>>>(
        A, reinterpret_cast<const unsigned long long *>(d_partials));
    c.launches++;
    e = cudaGetLastError();
    return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "key switch final launch");
}

int launch_lwe_keyswitch32_indexed(Context &c, const uint32_t *d_extract, size_t count, bool modswitch,
                                   uint64_t *d_out, const uint32_t *d_out_idx, cudaStream_t st)
{
    if (!count) return FHEACC_OK;
    if (!c.d_kskey) return c.fail(FHEACC_ENOKEY, "LWE key-switch key not uploaded");
    if (c.p.n + 1 > 4 * kKsMaxThreads) return c.fail(FHEACC_EINVAL, "n too large for key switch");
    dev::KsArgs A{};
    A.ext = d_extract; A.count = count; A.kskey = c.d_kskey; A.out = d_out; A.out_idx = d_out_idx;
    A.n = c.p.n; A.N = c.p.N; A.digitKS = (int)c.p.digitKS; A.Bks = c.p.Bks; A.ks_row = c.dp.ks_row;
    A.q = c.p.q; A.modswitch = modswitch ? 1u : 0u; A.Q = c.p.Q;
    const size_t smem = (size_t)c.p.N * c.p.digitKS;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device);
    const unsigned threads = (unsigned)(c.dp.ks_row / 4);   // ks_row: multiple of 32 words, > n
    size_t blocks = std::min<size_t>(count, (size_t)std::max(sms, 1) * 16);
    dev::lwe_ks32_kernel<<<(unsigned)blocks, threads, smem, st>>>(A);
    c.launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "lwe_ks32 launch");
}

int launch_modswitch(Context &c, const uint64_t *d_in, size_t count, uint64_t *d_out, cudaStream_t st)
{
    if (!count) return FHEACC_OK;
    size_t words = count * ((size_t)c.p.n + 1);
    unsigned blocks = (unsigned)std::min<size_t>((words + 255) / 256, 4096);
    dev::modswitch_kernel<<<blocks, 256, 0, st>>>(d_in, d_out, words, c.p.q, c.p.Q);
    c.launches++;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "modswitch launch");
}

}  // namespace fheacc
