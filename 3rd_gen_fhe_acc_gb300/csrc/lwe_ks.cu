// lwe_ks.cu -- RLWE -> LWE key switch and modulus switch: the 32-bit words'
// kernels, and the tiled form of both word widths (the 64-bit per-gate and
// split forms are in bootstrap64.cu).
//
// Reference behaviour: LWE::LWE_keyswitch (FHE_ACC_runtime/src/LWE.cpp:233-253)
// and LWE::LWE_modswitch / scale_round (LWE.cpp:255-269). The reference's FPGA
// path runs these on the host (myfpga.cpp:1519-1523); here they run on the GPU
// right after the blind rotation.
//
// Input is the extracted RLWE (time-domain a[N] after NTT_a_transpose, and
// b[0]). For every coefficient i < N and digit j < digitKS the LWE row
// kskey[d][j][i], d = base-Bks digit j of a[i], is subtracted.
//
// Batches of 1024 gates and more take the tiled form (lwe_ks32_tiled_kernel;
// 64-bit words from two gates per SM, lwe_ks64_tiled_kernel):
// ks_digits_kernel first writes every gate's digits gate-minor,
// [(i * digitKS + j)][gate]; then a CTA takes a block of gates and a 512-byte
// slice of the key rows and walks the N * digitKS row groups (the
// Bks rows of one (i, j)) in order, staging each group's row slices (and the
// block's digits) in shared memory with cp.async, several groups ahead, while
// each warp adds the slice its gates select. A row group is then read from L2
// once per gate block instead of once per gate (4096 gates: 32 blocks, the
// 315 MB key 32 times instead of 4096), and because every CTA walks the groups
// in the same order the key streams from HBM about once.
//
// Smaller batches: one CTA per ciphertext, the digits computed once into
// shared memory, then the CTA walks the N * digitKS rows; a row is n+1
// consecutive words, read by consecutive threads (coalesced). Below two gates
// per SM each gate's rows are split over many CTAs (ks_partial_kernel).
// Sums are kept in 64-bit registers without reduction (N * digitKS * Q <
// 2^64) and reduced once at the end; the modulus switch is fused into the
// same epilogue.
#include "ctx.hpp"
#include <algorithm>
#include <type_traits>

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
        A.out[(A.out_idx ? (size_t)A.out_idx[ci] : ci) * w + k] = A.modswitch ? scale_round_dev(v, A.q, A.Q) : v;
    }
}

// ---- tiled form

constexpr int kKsTileWarps = 16;   // warps of a tiled CTA
constexpr int kKsTileCols = 128;   // key-row words per CTA (4 per lane)
constexpr int kKsTileStages = 4;   // stages in flight (cp.async ring)
constexpr int kKsTileGroups = 2;   // row groups per stage (one barrier per stage)

struct KsTiledArgs {
    KsArgs k;                // 64-bit words: kskey and ks_row in 32-bit units (a u64 row is 2 ks_row words)
    const uint8_t *digits;   // [(i * digitKS + j)][gstride]: digit j of a[i] of each gate (ks_digit_slot)
    size_t gstride;          // bytes per digit row: 128 per gate block (64-bit words: 16 GW)
    int slices;              // column slices of kKsTileCols 32-bit words
    const uint64_t *ext64;   // 64-bit words: extracted RLWEs (kExtract64 words each)
};

// The digits of a gate block as the tiled kernel reads them: warp w of the
// block owns gates w GW .. w GW + GW - 1 and their digits of one row group sit
// in the warp's 8-byte slot, so a block's digits of a row group are 128 bytes
// (16 warps x 8) and a warp reads its own in one aligned 64-bit load.
__host__ __device__ __forceinline__ size_t ks_digit_slot(size_t g, int GW)
{
    const size_t G = (size_t)kKsTileWarps * GW, b = g / G, r = g - b * G;
    return b * (kKsTileWarps * 8) + (r / GW) * 8 + r % GW;
}

// digits[(i * D + j) * gstride + slot(g)] = (a_i / Bks^j) mod Bks of gate g
// (0 for the gates >= count of the last block). A CTA of 32 x 8 threads
// handles 32 gates x 32 coefficients: the extracted words are read row-wise
// (coalesced), transposed in shared memory, and each digit row is written 32
// gates at a time.
__global__ void __launch_bounds__(256) ks_digits_kernel(const uint32_t *__restrict__ ext, size_t count,
                                                        size_t padded, uint8_t *__restrict__ digits, size_t gstride,
                                                        int D, uint32_t Bks, int GW)
{
    __shared__ uint32_t tile[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const size_t g0 = (size_t)blockIdx.x * 32;
    const int i0 = blockIdx.y * 32;
#pragma unroll
    for (int r = 0; r < 4; r++) {
        const size_t g = g0 + ty + 8 * r;
        tile[ty + 8 * r][tx] = g < count ? ext[g * kExtractStride + i0 + tx] : 0u;
    }
    __syncthreads();
    const size_t g = g0 + tx;
    if (g >= padded) return;
    const size_t slot = ks_digit_slot(g, GW);
#pragma unroll
    for (int r = 0; r < 4; r++) {
        const int ci = ty + 8 * r;
        uint32_t a = tile[tx][ci];
        uint8_t *dst = digits + (size_t)(i0 + ci) * D * gstride + slot;
        for (int j = 0; j < D; j++) {
            dst[(size_t)j * gstride] = (uint8_t)(a % Bks);
            a /= Bks;
        }
    }
}

// 64-bit words: digits[(i * D + j) * gstride + g] = (a_i / Bks^j) mod Bks of
// gate g, the gates of a block contiguous (16 GW bytes per block and row
// group). Same 32 x 32 transpose as ks_digits_kernel. The quotients come from
// magic = ceil(2^64 / Bks): floor(a magic / 2^64) = floor(a / Bks) for every
// a below Q (the launcher checks Q (magic Bks - 2^64) < 2^64).
__global__ void __launch_bounds__(256) ks_digits64_kernel(const uint64_t *__restrict__ ext, size_t count,
                                                          size_t padded, uint8_t *__restrict__ digits, size_t gstride,
                                                          int D, uint32_t Bks, uint64_t magic)
{
    __shared__ uint64_t tile[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const size_t g0 = (size_t)blockIdx.x * 32;
    const int i0 = blockIdx.y * 32;
#pragma unroll
    for (int r = 0; r < 4; r++) {
        const size_t g = g0 + ty + 8 * r;
        tile[ty + 8 * r][tx] = g < count ? ext[g * kExtract64 + i0 + tx] : 0ull;
    }
    __syncthreads();
    const size_t g = g0 + tx;
    if (g >= padded) return;
#pragma unroll
    for (int r = 0; r < 4; r++) {
        const int ci = ty + 8 * r;
        uint64_t a = tile[tx][ci];
        uint8_t *dst = digits + (size_t)(i0 + ci) * D * gstride + g;
        for (int j = 0; j < D; j++) {
            const uint64_t qt = __umul64hi(a, magic);
            dst[(size_t)j * gstride] = (uint8_t)(a - qt * Bks);
            a = qt;
        }
    }
}

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int PENDING>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(PENDING) : "memory"); }

// CTA (gate block b, column slice s): gates [b G, b G + G), G = 16 GW, key
// words [s 128, s 128 + 128) (32-bit units: 64 words of a 64-bit row). The row
// groups are walked kKsTileGroups at a time: a stage of the ring holds that
// many groups' Bks row slices ([Bks][512 bytes] each) and the block's digit
// bytes of each group. Every thread copies the same chunks of every stage;
// their source addresses move by a per-group offset that is advanced, not
// recomputed. Warp w owns gates w GW .. w GW + GW - 1 and lane l the 16 bytes
// 16 l .. 16 l + 15 of the slice: per row group it reads its gates' digits and
// adds, for each gate, the row slice the digit selects (one 128-bit shared
// load; all lanes read one row, so a warp's load is 512 contiguous bytes, free
// of bank conflicts). Sums stay below 32 Q with a conditional subtraction of
// 16 Q every 16 row groups (rows are canonical): 32-bit sums for Q < 2^27,
// 64-bit sums for the 64-bit words.
// 32-bit words: GW <= 8, the block's digits of a group in 8-byte slots per
// warp (ks_digit_slot), read in one 64-bit load. 64-bit words (WIDE): GW <=
// 16, the block's G digit bytes contiguous, read as bytes.
template <int GW, bool WIDE>
__device__ __forceinline__ void ks_tiled_body(const KsTiledArgs &T, uint32_t *ring)
{
    constexpr int R = kKsTileGroups;
    constexpr int kMaxChunks = 4;   // chunks of a stage per thread (checked by the launcher)
    constexpr int kDigitBytes = WIDE ? kKsTileWarps * GW : kKsTileWarps * 8;   // per block and row group
    constexpr int kDigitWords = kDigitBytes / 4;
    using Acc = typename std::conditional<WIDE, uint64_t, uint32_t>::type;
    constexpr int AE = WIDE ? 2 : 4;   // sums per gate and lane
    const KsArgs &A = T.k;
    const int N = A.N, D = A.digitKS, Bks = (int)A.Bks, n = A.n;
    const int group_words = Bks * kKsTileCols + kDigitWords;   // row slices, then digit slots
    const int group_chunks = group_words / 4, rows_chunks = Bks * (kKsTileCols / 4);
    const int stage_words = R * group_words;
    const int slice = blockIdx.x % T.slices;
    const size_t gb = blockIdx.x / T.slices;
    const size_t g0 = gb * (kKsTileWarps * GW);
    const int c0 = slice * kKsTileCols;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const Acc Q = (Acc)A.Q, Q16 = 16 * Q;
    const int total = N * D;
    const size_t row_stride = (size_t)D * N * A.ks_row;   // words between digits d and d + 1

    // this thread's chunks: their group of the stage, source pointer for stage
    // 0 (rows: kskey row (d, j, i) slice; digits: the block's slots) and
    // destination word in the stage
    const char *src[kMaxChunks];
    int dst[kMaxChunks], grp[kMaxChunks];
    bool dig[kMaxChunks];
#pragma unroll
    for (int u = 0; u < kMaxChunks; u++) {
        const int c = threadIdx.x + u * (int)blockDim.x;
        src[u] = nullptr;
        dst[u] = 0;
        grp[u] = -1;
        dig[u] = false;
        if (c < R * group_chunks) {
            const int r = c / group_chunks, cc = c - r * group_chunks;
            grp[u] = r;
            dst[u] = r * group_words + 4 * cc;
            // row group r of stage 0: (i, j) = (r / D, r % D)
            const int i = r / D, j = r - (r / D) * D;
            if (cc < rows_chunks) {
                src[u] = reinterpret_cast<const char *>(A.kskey + ((size_t)j * N + i) * A.ks_row + c0 +
                                                        (size_t)(cc >> 5) * row_stride + 4 * (cc & 31));
            } else {
                dig[u] = true;
                src[u] = reinterpret_cast<const char *>(T.digits + (size_t)r * T.gstride + gb * kDigitBytes +
                                                        16 * (cc - rows_chunks));
            }
        }
    }
    // per group of the next stage to fetch: its (i, j), to advance the row offsets
    int gi[R], gj[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
        gi[r] = r / D;
        gj[r] = r - gi[r] * D;
    }
    int fetched = 0;   // row groups issued so far
    auto issue_stage = [&]() {
        uint32_t *ring_stage = ring + ((fetched / R) % kKsTileStages) * stage_words;
#pragma unroll
        for (int u = 0; u < kMaxChunks; u++)
            if (grp[u] >= 0 && fetched + grp[u] < total) cp_async16(ring_stage + dst[u], src[u]);
        // advance every group by R row groups: the rows by the change of (i, j),
        // the digits by R rows of slots
        long long drow[R];
#pragma unroll
        for (int r = 0; r < R; r++) {
            const long long before = (long long)gj[r] * N + gi[r];
            gj[r] += R;
            while (gj[r] >= D) {
                gj[r] -= D;
                gi[r]++;
            }
            drow[r] = ((long long)gj[r] * N + gi[r] - before) * (long long)A.ks_row * 4;
        }
#pragma unroll
        for (int u = 0; u < kMaxChunks; u++) {
            long long d = dig[u] ? (long long)R * (long long)T.gstride : 0;
#pragma unroll
            for (int r = 0; r < R; r++)
                if (!dig[u] && grp[u] == r) d = drow[r];
            src[u] += d;
        }
        fetched += R;
    };

#pragma unroll
    for (int s = 0; s < kKsTileStages - 1; s++) {
        if (fetched < total) issue_stage();
        cp_async_commit();
    }
    Acc acc[GW][AE];
#pragma unroll
    for (int k = 0; k < GW; k++)
#pragma unroll
        for (int e = 0; e < AE; e++) acc[k][e] = 0;

    for (int rg = 0; rg < total; rg += R) {
        cp_async_wait<kKsTileStages - 2>();
        __syncthreads();
        // the stage read in the previous iteration is free: fetch ahead into it
        if (fetched < total) issue_stage();
        cp_async_commit();
        const uint32_t *st = ring + ((rg / R) % kKsTileStages) * stage_words;
#pragma unroll
        for (int r = 0; r < R; r++) {
            if (rg + r < total) {
                const uint32_t *grp_w = st + r * group_words;
                const uint4 *rows4 = reinterpret_cast<const uint4 *>(grp_w);
                if constexpr (!WIDE) {
                    const uint2 dg2 = reinterpret_cast<const uint2 *>(grp_w + Bks * kKsTileCols)[warp];
#pragma unroll
                    for (int k = 0; k < GW; k++) {
                        const uint32_t d = ((k < 4 ? dg2.x : dg2.y) >> (8 * (k & 3))) & 0xFFu;
                        const uint4 v = rows4[d * (kKsTileCols / 4) + lane];
                        acc[k][0] += v.x;
                        acc[k][1] += v.y;
                        acc[k][2] += v.z;
                        acc[k][3] += v.w;
                    }
                } else {
                    const uint8_t *dgb = reinterpret_cast<const uint8_t *>(grp_w + Bks * kKsTileCols) + warp * GW;
#pragma unroll
                    for (int k = 0; k < GW; k++) {
                        const uint32_t d = dgb[k];
                        const ulonglong2 v = reinterpret_cast<const ulonglong2 *>(rows4)[d * (kKsTileCols / 4) + lane];
                        acc[k][0] += v.x;
                        acc[k][1] += v.y;
                    }
                }
            }
        }
        if (((rg / R) & (16 / R - 1)) == 16 / R - 1) {
#pragma unroll
            for (int k = 0; k < GW; k++)
#pragma unroll
                for (int e = 0; e < AE; e++) acc[k][e] = min(acc[k][e], acc[k][e] - Q16);
        }
    }
    cp_async_wait<0>();

    const Acc Q8 = Q / 8 + 1;
#pragma unroll
    for (int k = 0; k < GW; k++) {
        const size_t g = g0 + warp * GW + k;
        if (g >= A.count) continue;
        const Acc b0 = WIDE ? (Acc)T.ext64[g * kExtract64 + N] : (Acc)A.ext[g * kExtractStride + N];
        uint64_t *out = A.out + (A.out_idx ? (size_t)A.out_idx[g] : g) * (size_t)(n + 1);
#pragma unroll
        for (int e = 0; e < AE; e++) {
            const int col = (WIDE ? c0 / 2 + 2 * lane : c0 + 4 * lane) + e;
            if (col > n) continue;
            const Acc s = acc[k][e] % Q;
            uint64_t v;
            if (col < n) v = s ? Q - s : 0;
            else v = ((uint64_t)(b0 + Q8) % Q + Q - s) % Q;
            out[col] = A.modswitch ? scale_round_dev(v, A.q, A.Q) : v;
        }
    }
}

template <int GW>
__global__ void __launch_bounds__(kKsTileWarps * 32, 1) lwe_ks32_tiled_kernel(const __grid_constant__ KsTiledArgs T)
{
    extern __shared__ __align__(16) uint32_t ring[];
    ks_tiled_body<GW, false>(T, ring);
}

// The tiled form for 64-bit words (N = 2048, Q < 2^58): same staging, 64-bit
// sums, gates per warp up to 16.
template <int GW>
__global__ void __launch_bounds__(kKsTileWarps * 32, 1) lwe_ks64_tiled_kernel(const __grid_constant__ KsTiledArgs T)
{
    extern __shared__ __align__(16) uint32_t ring[];
    ks_tiled_body<GW, true>(T, ring);
}

__global__ void modswitch_kernel(const uint64_t *__restrict__ in, uint64_t *__restrict__ out, size_t words,
                                 uint64_t q, uint64_t Q)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < words; i += (size_t)gridDim.x * blockDim.x)
        out[i] = scale_round_dev(in[i], q, Q);
}

}  // namespace dev

template <int GW, bool WIDE = false>
static int launch_ks_tiled_gw(Context &c, const dev::KsTiledArgs &T, size_t blocks, size_t smem, cudaStream_t st)
{
    void (*kern)(const dev::KsTiledArgs);
    if constexpr (WIDE) kern = dev::lwe_ks64_tiled_kernel<GW>;
    else kern = dev::lwe_ks32_tiled_kernel<GW>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return c.cuda_fail(e, "tiled key switch smem attribute");
    kern<<<(unsigned)blocks, dev::kKsTileWarps * 32, smem, st>>>(T);
    c.launches++;
    e = cudaGetLastError();
    return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "tiled key switch launch");
}

// Gates per warp of the tiled form (1..8, the bytes of a warp's digit slot):
// gate blocks of 16 GW gates, the smallest GW with which the blocks times the
// column slices fit on the SMs (4096 gates: 7, 37 blocks x 4 slices = 148 CTAs).
static int ks_tiled_gw(size_t count, int sms, int slices)
{
    const size_t blocks_target = std::max<size_t>(1, (size_t)sms / slices);
    const size_t per_warp = ((count + blocks_target - 1) / blocks_target + dev::kKsTileWarps - 1) / dev::kKsTileWarps;
    return (int)std::min<size_t>(8, std::max<size_t>(1, per_warp));
}

// Scratch bytes the tiled key switch of `count` gates needs for its digits:
// 128 slot bytes per gate block and row group.
static size_t ks_tiled_digit_bytes(const Context &c, size_t count, int sms)
{
    const int slices = (int)(c.dp.ks_row / dev::kKsTileCols);
    const size_t G = (size_t)dev::kKsTileWarps * ks_tiled_gw(count, sms, std::max(slices, 1));
    return (count + G - 1) / G * (dev::kKsTileWarps * 8) * (size_t)c.p.N * c.p.digitKS;
}

static bool ks_tiled_applies(const Context &c, size_t count, int sms, size_t scratch_bytes)
{
    if (c.tune.ks_tiled == 0) return false;
    if (c.dp.ks_row % dev::kKsTileCols != 0 || c.p.N % 32 != 0 || c.p.Bks > 255) return false;
    // a thread copies at most 4 chunks of a stage
    if ((size_t)dev::kKsTileGroups * (c.p.Bks * (dev::kKsTileCols / 4) + 8) > 4 * 32 * (size_t)dev::kKsTileWarps)
        return false;
    if (ks_tiled_digit_bytes(c, count, sms) > scratch_bytes) return false;
    if (c.tune.ks_tiled > 0) return true;
    return count >= kKsTiledMinGates;
}

static int launch_ks_tiled(Context &c, const dev::KsArgs &A, void *scratch, int sms, cudaStream_t st)
{
    const int slices = (int)(c.dp.ks_row / dev::kKsTileCols);
    const int GW = ks_tiled_gw(A.count, sms, slices);
    const size_t G = (size_t)dev::kKsTileWarps * GW, nblocks = (A.count + G - 1) / G;
    dev::KsTiledArgs T{};
    T.k = A;
    T.digits = (const uint8_t *)scratch;
    T.gstride = nblocks * (dev::kKsTileWarps * 8);
    T.slices = slices;
    const size_t padded = nblocks * G;
    dim3 dgrid((unsigned)((padded + 31) / 32), (unsigned)(c.p.N / 32));
    dev::ks_digits_kernel<<<dgrid, 256, 0, st>>>(A.ext, A.count, padded, (uint8_t *)scratch, T.gstride,
                                                 A.digitKS, A.Bks, GW);
    c.launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return c.cuda_fail(e, "key-switch digits launch");
    const size_t blocks = nblocks * slices;
    const size_t smem = (size_t)dev::kKsTileStages * dev::kKsTileGroups *
                        ((size_t)c.p.Bks * dev::kKsTileCols + dev::kKsTileWarps * 2) * sizeof(uint32_t);
    switch (GW) {
    case 1: return launch_ks_tiled_gw<1>(c, T, blocks, smem, st);
    case 2: return launch_ks_tiled_gw<2>(c, T, blocks, smem, st);
    case 3: return launch_ks_tiled_gw<3>(c, T, blocks, smem, st);
    case 4: return launch_ks_tiled_gw<4>(c, T, blocks, smem, st);
    case 5: return launch_ks_tiled_gw<5>(c, T, blocks, smem, st);
    case 6: return launch_ks_tiled_gw<6>(c, T, blocks, smem, st);
    case 7: return launch_ks_tiled_gw<7>(c, T, blocks, smem, st);
    default: return launch_ks_tiled_gw<8>(c, T, blocks, smem, st);
    }
}

// ---- tiled form of the 64-bit words (lwe_ks64_tiled_kernel)

// Gates per warp (1..16): the smallest with which the gate blocks times the
// column slices fit on the SMs (2048 gates at N = 2048, n = 630: 9 gates per
// warp, 15 blocks x 10 slices = 150 CTAs).
static int ks64_tiled_gw(size_t count, int sms, int slices)
{
    const size_t blocks_target = std::max<size_t>(1, (size_t)sms / slices);
    const size_t per_warp = ((count + blocks_target - 1) / blocks_target + dev::kKsTileWarps - 1) / dev::kKsTileWarps;
    return (int)std::min<size_t>(16, std::max<size_t>(1, per_warp));
}

// ceil(2^64 / Bks), the digits kernel's quotient multiplier; 0 if its
// quotients are not exact for every word below Q.
static uint64_t ks64_digit_magic(const Context &c)
{
    const uint64_t B = c.p.Bks;
    if (B < 2) return 0;
    const uint64_t m = UINT64_MAX / B + 1;
    const unsigned __int128 err = (unsigned __int128)m * B - ((unsigned __int128)1 << 64);   // in [0, B)
    return (unsigned __int128)c.p.Q * err < ((unsigned __int128)1 << 64) ? m : 0;
}

bool ks64_tiled_applies(const Context &c, size_t count, int sms, size_t scratch_bytes)
{
    if (c.tune.ks_tiled == 0) return false;
    const int slices = (int)(2 * c.dp.ks_row / dev::kKsTileCols);
    if ((2 * c.dp.ks_row) % dev::kKsTileCols != 0 || c.p.N % 32 != 0 || c.p.Bks > 255 || !ks64_digit_magic(c))
        return false;
    // a thread copies at most 4 chunks of a stage (16 digit chunks at most)
    if ((size_t)dev::kKsTileGroups * (c.p.Bks * (dev::kKsTileCols / 4) + 16) > 4 * 32 * (size_t)dev::kKsTileWarps)
        return false;
    const size_t G = (size_t)dev::kKsTileWarps * ks64_tiled_gw(count, sms, slices);
    if ((count + G - 1) / G * G * (size_t)c.p.N * c.p.digitKS > scratch_bytes) return false;
    if (c.tune.ks_tiled > 0) return true;
    return count >= 2 * (size_t)sms;
}

// Runs the tiled 64-bit key switch (ks64_tiled_applies must hold): the digits
// into `scratch`, then lwe_ks64_tiled_kernel.
int launch_ks64_tiled(Context &c, const uint64_t *d_extract, size_t count, bool modswitch, uint64_t *d_out,
                      const uint32_t *d_out_idx, void *scratch, int sms, cudaStream_t st)
{
    const int slices = (int)(2 * c.dp.ks_row / dev::kKsTileCols);
    const int GW = ks64_tiled_gw(count, sms, slices);
    const size_t G = (size_t)dev::kKsTileWarps * GW, nblocks = (count + G - 1) / G, padded = nblocks * G;
    dev::KsTiledArgs T{};
    T.k.ext = nullptr; T.k.count = count; T.k.kskey = reinterpret_cast<const uint32_t *>(c.d_kskey64);
    T.k.out = d_out; T.k.out_idx = d_out_idx;
    T.k.n = c.p.n; T.k.N = c.p.N; T.k.digitKS = (int)c.p.digitKS; T.k.Bks = c.p.Bks;
    T.k.ks_row = 2 * c.dp.ks_row;   // 32-bit words per 64-bit row
    T.k.q = c.p.q; T.k.modswitch = modswitch ? 1u : 0u; T.k.Q = c.p.Q;
    T.digits = (const uint8_t *)scratch;
    T.gstride = padded;
    T.slices = slices;
    T.ext64 = d_extract;
    dim3 dgrid((unsigned)((padded + 31) / 32), (unsigned)(c.p.N / 32));
    dev::ks_digits64_kernel<<<dgrid, 256, 0, st>>>(d_extract, count, padded, (uint8_t *)scratch, T.gstride,
                                                   (int)c.p.digitKS, c.p.Bks, ks64_digit_magic(c));
    c.launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return c.cuda_fail(e, "key-switch digits launch");
    const size_t blocks = nblocks * slices;
    const size_t smem = (size_t)dev::kKsTileStages * dev::kKsTileGroups *
                        ((size_t)c.p.Bks * dev::kKsTileCols + 4 * (size_t)GW) * sizeof(uint32_t);
    switch (GW) {
    case 1: return launch_ks_tiled_gw<1, true>(c, T, blocks, smem, st);
    case 2: return launch_ks_tiled_gw<2, true>(c, T, blocks, smem, st);
    case 3: return launch_ks_tiled_gw<3, true>(c, T, blocks, smem, st);
    case 4: return launch_ks_tiled_gw<4, true>(c, T, blocks, smem, st);
    case 5: return launch_ks_tiled_gw<5, true>(c, T, blocks, smem, st);
    case 6: return launch_ks_tiled_gw<6, true>(c, T, blocks, smem, st);
    case 7: return launch_ks_tiled_gw<7, true>(c, T, blocks, smem, st);
    case 8: return launch_ks_tiled_gw<8, true>(c, T, blocks, smem, st);
    case 9: return launch_ks_tiled_gw<9, true>(c, T, blocks, smem, st);
    case 10: return launch_ks_tiled_gw<10, true>(c, T, blocks, smem, st);
    case 11: return launch_ks_tiled_gw<11, true>(c, T, blocks, smem, st);
    case 12: return launch_ks_tiled_gw<12, true>(c, T, blocks, smem, st);
    case 13: return launch_ks_tiled_gw<13, true>(c, T, blocks, smem, st);
    case 14: return launch_ks_tiled_gw<14, true>(c, T, blocks, smem, st);
    case 15: return launch_ks_tiled_gw<15, true>(c, T, blocks, smem, st);
    default: return launch_ks_tiled_gw<16, true>(c, T, blocks, smem, st);
    }
}

int launch_lwe_keyswitch32(Context &c, const uint32_t *d_extract, size_t count, bool modswitch, uint64_t *d_out,
                           cudaStream_t st, void *d_scratch, size_t scratch_bytes, const uint32_t *d_out_idx)
{
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.device);
    sms = std::max(sms, 1);
    if (!count) return FHEACC_OK;
    if (!c.d_kskey) return c.fail(FHEACC_ENOKEY, "LWE key-switch key not uploaded");
    if (c.p.n + 1 > 4 * kKsMaxThreads) return c.fail(FHEACC_EINVAL, "n too large for key switch");
    dev::KsArgs A{};
    A.ext = d_extract; A.count = count; A.kskey = c.d_kskey; A.out = d_out; A.out_idx = d_out_idx;
    A.n = c.p.n; A.N = c.p.N; A.digitKS = (int)c.p.digitKS; A.Bks = c.p.Bks; A.ks_row = c.dp.ks_row;
    A.q = c.p.q; A.modswitch = modswitch ? 1u : 0u; A.Q = c.p.Q;
    if (d_scratch && ks_tiled_applies(c, count, sms, scratch_bytes)) return launch_ks_tiled(c, A, d_scratch, sms, st);
    // a few ciphertexts: split each one's rows over many CTAs
    if (!d_scratch || count >= 2 * (size_t)sms || count * c.dp.ks_row * sizeof(uint64_t) > scratch_bytes)
        return launch_lwe_keyswitch32_indexed(c, d_extract, count, modswitch, d_out, d_out_idx, st);
    uint64_t *d_partials = (uint64_t *)d_scratch;
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
