// api.cu -- the C ABI of libfheacc.so (declared in include/fheacc.h): device
// context, key upload with the one-time device re-layout, and the bootstrap
// entry points. Replaces the FPGA backend's configuration, DMA and issue loop
// (FHE_ACC_runtime/src/myfpga.cpp:82-1660).
#include "ctx.hpp"
#include "host/host_math.hpp"
#include <algorithm>
#include <chrono>
#include <cstring>
#include <new>
#include <thread>
#include <vector>

using namespace fheacc;

static thread_local std::string g_create_error;

namespace fheacc {

int ensure_scratch(Context &c, Scratch &s, size_t bytes)
{
    if (s.bytes >= bytes) return FHEACC_OK;
    if (s.ptr) {
        cudaStreamSynchronize(c.stream);
        cudaFree(s.ptr);   // implicit device synchronisation
        s.ptr = nullptr;
        s.bytes = 0;
    }
    size_t want = std::max(bytes, (size_t)1 << 20);
    cudaError_t e = cudaMalloc(&s.ptr, want);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return c.fail(FHEACC_ENOMEM, std::string("scratch allocation failed: ") + cudaGetErrorString(e));
    }
    s.bytes = want;
    return FHEACC_OK;
}

// Reads and clears the device status word after the context's work finished;
// a set bit means a kernel abandoned a bounded wait and its results are invalid.
static int take_device_status(Context &c, uint32_t *bits)
{
    uint32_t v = 0;
    cudaError_t e = cudaMemcpy(&v, c.d_status, sizeof(v), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && v) e = cudaMemset(c.d_status, 0, sizeof(v));
    if (e != cudaSuccess) return c.cuda_fail(e, "device status");
    if (bits) *bits = v;
    if (v & kStatusWaitLimit)
        return c.fail(FHEACC_EIO, "a blind-rotation worker gave up a bounded wait on another worker; results invalid");
    return FHEACC_OK;
}

int prepare_window(Context &c, int steps, cudaStream_t st, dev::StepWindow &w)
{
    w = dev::StepWindow{};
    const int K = c.tune.br_window < 0 ? kWindowWide : c.tune.br_window;
    if (K <= 0 || !c.d_window || steps <= 0) return FHEACC_OK;
    const int buckets = (steps + K - 1) / K;
    if (buckets > kWindowCapacity) return FHEACC_OK;
    cudaError_t e = cudaMemsetAsync(c.d_window, 0, (buckets + 1) * sizeof(unsigned), st);
    if (e != cudaSuccess) return c.cuda_fail(e, "step-window reset");
    w.count = c.d_window;
    w.steps = K;
    w.buckets = buckets;
    // a bucket of the slowest CTAs takes well under a millisecond (32-bit) or a
    // few milliseconds (64-bit); CTAs stop waiting after about 10 / 40 ms
    w.spin_limit = c.tune.debug_wait_limit >= 0 ? (unsigned)c.tune.debug_wait_limit : c.wide ? 160000u : 40000u;
    return FHEACC_OK;
}


int bootstrap_device_with(Context &c, const uint64_t *d_c1, const uint64_t *d_c2, const int32_t *d_gates,
                          size_t count, uint64_t *d_out, uint32_t flags, void *accs, void *extract,
                          cudaStream_t st)
{
    flags &= ~(uint32_t)FHEACC_FLAG_PROFILE;
    if (c.wide) {
        if (!c.d_btkey64) return c.fail(FHEACC_ENOKEY, "bootstrap key not uploaded");
        if (!c.d_kskey64) return c.fail(FHEACC_ENOKEY, "LWE key-switch key not uploaded");
        int rc = launch_blind_rotate64_with(c, d_c1, d_c2, d_gates, count, flags, (uint64_t *)accs, nullptr,
                                            (uint64_t *)extract, 0, st);
        return rc ? rc : launch_lwe_keyswitch64(c, (const uint64_t *)extract, count, true, d_out, st, nullptr, accs,
                                                bootstrap_accs_bytes(c, count));
    }
    if (!c.d_btkey) return c.fail(FHEACC_ENOKEY, "bootstrap key not uploaded");
    if (!c.d_kskey) return c.fail(FHEACC_ENOKEY, "LWE key-switch key not uploaded");
    int rc = launch_blind_rotate32_with(c, d_c1, d_c2, d_gates, count, flags, (uint32_t *)accs, (uint32_t *)extract,
                                        st);
    // the accumulators are free once the blind rotation is done
    return rc ? rc : launch_lwe_keyswitch32(c, (const uint32_t *)extract, count, true, d_out, st, accs,
                                            bootstrap_accs_bytes(c, count));
}

int bootstrap_device(Context &c, const uint64_t *d_c1, const uint64_t *d_c2, const int32_t *d_gates,
                     size_t count, uint64_t *d_out, uint32_t flags, cudaStream_t st, int max_ctas)
{
    if (c.wide) {
        if (!c.d_btkey64) return c.fail(FHEACC_ENOKEY, "bootstrap key not uploaded");
        if (!c.d_kskey64) return c.fail(FHEACC_ENOKEY, "LWE key-switch key not uploaded");
        int rc = ensure_scratch(c, c.extract, count * kExtract64 * sizeof(uint64_t));
        if (rc) return rc;
        uint64_t *ext = (uint64_t *)c.extract.ptr;
        const bool prof = (flags & FHEACC_FLAG_PROFILE) != 0;
        if (prof) cudaEventRecord(c.prof[0], st);
        rc = launch_blind_rotate64(c, d_c1, d_c2, d_gates, count, flags, nullptr, ext, max_ctas, st);
        if (rc) return rc;
        if (prof) cudaEventRecord(c.prof[1], st);
        rc = launch_lwe_keyswitch64(c, ext, count, true, d_out, st, nullptr, c.accs.ptr, c.accs.bytes);
        if (prof && rc == FHEACC_OK) cudaEventRecord(c.prof[2], st);
        return rc;
    }
    if (!c.d_btkey) return c.fail(FHEACC_ENOKEY, "bootstrap key not uploaded");
    if (!c.d_kskey) return c.fail(FHEACC_ENOKEY, "LWE key-switch key not uploaded");
    int rc = ensure_scratch(c, c.extract, count * kExtractStride * sizeof(uint32_t));
    if (rc) return rc;
    uint32_t *ext = (uint32_t *)c.extract.ptr;
    const bool prof = (flags & FHEACC_FLAG_PROFILE) != 0;
    if (prof) cudaEventRecord(c.prof[0], st);
    rc = launch_blind_rotate32(c, d_c1, d_c2, d_gates, count, flags, nullptr, ext, max_ctas, st);
    if (rc) return rc;
    if (prof) cudaEventRecord(c.prof[1], st);
    // the accumulator scratch is free once the blind rotation is done
    rc = launch_lwe_keyswitch32(c, ext, count, true, d_out, st, c.accs.ptr, c.accs.bytes);
    if (prof && rc == FHEACC_OK) cudaEventRecord(c.prof[2], st);
    return rc;
}

}  // namespace fheacc

namespace {

// NULL selects the legacy default stream, as in the CUDA runtime API.
cudaStream_t pick_stream(Context *, void *stream) { return (cudaStream_t)stream; }

// Marks the end of an asynchronous call so that fheacc_sync can wait for it.
int mark_done(Context &c, cudaStream_t st, int rc)
{
    if (rc != FHEACC_OK) return rc;
    cudaError_t e = cudaEventRecord(c.done, st);
    return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "event record");
}

uint32_t shoup32_companion(uint64_t w, uint64_t Q) { return (uint32_t)((w << 32) / Q); }

uint64_t shoup64_companion(uint64_t w, uint64_t Q) { return (uint64_t)(((unsigned __int128)w << 64) / Q); }

int build_tables64(Context &c)
{
    host::Tables T;
    T.build(c.p);
    const int N = c.p.N;
    const uint64_t Q = c.p.Q;
    std::vector<ulonglong2> fw(N), iw(N);
    for (int i = 0; i < N; i++) {
        fw[i] = make_ulonglong2(T.rou[i], shoup64_companion(T.rou[i], Q));
        iw[i] = make_ulonglong2(T.irou[i], shoup64_companion(T.irou[i], Q));
    }
    cudaError_t e = cudaMalloc(&c.d_tw64, N * sizeof(ulonglong2));
    if (e == cudaSuccess) e = cudaMalloc(&c.d_itw64, N * sizeof(ulonglong2));
    if (e == cudaSuccess) e = cudaMemcpy(c.d_tw64, fw.data(), N * sizeof(ulonglong2), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(c.d_itw64, iw.data(), N * sizeof(ulonglong2), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return c.cuda_fail(e, "twiddle upload");
    dev::Ntt64Consts &k = c.nc64;
    k.Q = Q;
    k.twoQ = 2 * Q;
    k.iN = c.p.iN;
    k.iNs = shoup64_companion(c.p.iN, Q);
    k.iw1N = host::mulmod(T.irou[1], c.p.iN, Q);
    k.iw1Ns = shoup64_companion(k.iw1N, Q);
    k.mu64 = c.dp.mu64;
    // factors of the last-digit identity (DevParams::last_digit_from_acc), for
    // the bootstrap key and for every RGSW a RLWE x RGSW product takes:
    // BG^(h - digitG + 1) for h < digitG - 1, BG^-(digitG - 1) for the last row
    const uint64_t dG = c.p.digitG;
    const uint64_t bg_inv = host::powmod(((uint64_t)1 << c.p.BG_bits) % Q, Q - 2, Q);
    std::vector<ulonglong2> cf(dG);
    for (uint64_t h = 0; h < dG; h++) {
        const uint64_t f = host::powmod(bg_inv, h + 1 < dG ? dG - 1 - h : dG - 1, Q);
        cf[h] = make_ulonglong2(f, shoup64_companion(f, Q));
    }
    e = cudaMalloc(&c.d_cf64, dG * sizeof(ulonglong2));
    if (e == cudaSuccess) e = cudaMemcpy(c.d_cf64, cf.data(), dG * sizeof(ulonglong2), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return c.cuda_fail(e, "key factors");
    return FHEACC_OK;
}

int build_tables(Context &c)
{
    if (c.wide) return build_tables64(c);
    host::Tables T;
    T.build(c.p);
    const int N = c.p.N;
    const uint64_t Q = c.p.Q;
    // Lane-interleaved per-lane twiddles of the layout-B NTT stages (see
    // load_stage_twiddles in ntt32.cuh): entry m + G*lane + g at
    // off + (g/2)*64 + 2*lane + g%2.
    std::vector<uint2> fw(N, make_uint2(0, 0)), iw(N, make_uint2(0, 0));
    auto put = [&](std::vector<uint2> &dst, const std::vector<uint64_t> &tab, int off, int m, int G) {
        for (int lane = 0; lane < 32; lane++)
            for (int g = 0; g < G; g++) {
                const uint64_t w = tab[m + G * lane + g];
                const int at = G == 1 ? off + lane : off + (g / 2) * 64 + 2 * lane + (g % 2);
                dst[at] = make_uint2((uint32_t)w, shoup32_companion(w, Q));
            }
    };
    for (int s = 5; s <= 9; s++) put(fw, T.rou, 32 * ((1 << (s - 5)) - 1), 1 << s, 16 >> (9 - s));
    for (int t = 1; t <= 16; t *= 2) put(iw, T.irou, 32 * (32 - 32 / t), 512 / t, 16 / t);
    cudaError_t e = cudaMalloc(&c.d_fwd_tw, N * sizeof(uint2));
    if (e == cudaSuccess) e = cudaMalloc(&c.d_inv_tw, N * sizeof(uint2));
    if (e == cudaSuccess) e = cudaMemcpy(c.d_fwd_tw, fw.data(), N * sizeof(uint2), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(c.d_inv_tw, iw.data(), N * sizeof(uint2), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return c.cuda_fail(e, "twiddle upload");
    dev::Ntt32Consts &k = c.nc;
    std::memset(&k, 0, sizeof k);
    k.Q = (uint32_t)Q;
    k.twoQ = (uint32_t)(2 * Q);
    for (int i = 1; i < 32; i++) {
        k.fw[i] = (uint32_t)T.rou[i];
        k.fws[i] = shoup32_companion(T.rou[i], Q);
        k.iw[i] = (uint32_t)T.irou[i];
        k.iws[i] = shoup32_companion(T.irou[i], Q);
    }
    k.iN = (uint32_t)c.p.iN;
    k.iNs = shoup32_companion(c.p.iN, Q);
    uint64_t w1 = host::mulmod(T.irou[1], c.p.iN, Q);
    k.iw1N = (uint32_t)w1;
    k.iw1Ns = shoup32_companion(w1, Q);
    return FHEACC_OK;
}

// NTT(-X^(N - 2^j)) for j < log2 N, as rotate_vector_gen(false) builds them
// (params.cpp:196-207); used by expand_RLWE's RLWE_rotate_freq.
int build_rotations(Context &c)
{
    host::Tables T;
    T.build(c.p);
    const int N = c.p.N, logN = T.logN;
    std::vector<uint64_t> rot((size_t)logN * N, 0), fwd((size_t)logN * N, 0);
    for (int j = 0; j < logN; j++) {
        uint64_t *v = rot.data() + (size_t)j * N;
        v[N - (1 << j)] = c.p.Q - 1;
        T.ntt(v);
        uint64_t *w = fwd.data() + (size_t)j * N;   // rotate_vector_gen(true): NTT(X^(2^j))
        w[1 << j] = 1;
        T.ntt(w);
    }
    cudaError_t e = cudaMalloc(&c.d_rot, rot.size() * sizeof(uint64_t));
    if (e == cudaSuccess) e = cudaMemcpy(c.d_rot, rot.data(), rot.size() * sizeof(uint64_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&c.d_rot_fwd, fwd.size() * sizeof(uint64_t));
    if (e == cudaSuccess)
        e = cudaMemcpy(c.d_rot_fwd, fwd.data(), fwd.size() * sizeof(uint64_t), cudaMemcpyHostToDevice);
    return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "rotation tables");
}

// Copies `words` 32-bit words from a host vector into device memory in chunks.
int upload_u32(Context &c, uint32_t *dst, const uint32_t *src, size_t words)
{
    cudaError_t e = cudaMemcpy(dst, src, words * sizeof(uint32_t), cudaMemcpyHostToDevice);
    return e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "key upload");
}

}  // namespace

extern "C" {

int fheacc_create(const fheacc_params *p, int device, fheacc_ctx **out)
{
    if (!p || !out) {
        g_create_error = "null argument";
        return FHEACC_EINVAL;
    }
    *out = nullptr;
    fheacc_params pp = *p;
    if (fheacc_params_derive(&pp) != FHEACC_OK) {
        const char *why = host::check_params(pp);
        g_create_error = std::string("invalid parameter set: ") + (why ? why : "derivation failed");
        return FHEACC_EINVAL;
    }
    const bool narrow = pp.N == 1024 && pp.Q < (1ULL << 27) && pp.digitG >= 2 && pp.digitG <= 4;
    const bool wide = pp.N == 2048 && pp.Q < (1ULL << 58) && pp.digitG >= 1 && pp.digitG <= 8;
    if (!narrow && !wide) {
        g_create_error = "unsupported parameter set: the device paths run N = 1024 with Q < 2^27 (digitG 2..4) "
                         "and N = 2048 with Q < 2^58 (digitG <= 8)";
        return FHEACC_EINVAL;
    }
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev <= 0 || device < 0 || device >= ndev) {
        cudaGetLastError();
        g_create_error = std::string("no usable CUDA device: ") + (e != cudaSuccess ? cudaGetErrorString(e) : "bad index");
        return FHEACC_ENODEV;
    }
    Context *c = new (std::nothrow) Context();
    if (!c) {
        g_create_error = "out of host memory";
        return FHEACC_ENOMEM;
    }
    c->p = pp;
    c->device = device;
    c->wide = wide;
    DeviceGuard g(device);
    DevParams &d = c->dp;
    d.n = pp.n; d.N = pp.N; d.logN = wide ? 11 : 10; d.q = pp.q; d.embed = 2u * (uint32_t)pp.N / pp.q; d.Q = pp.Q;
    d.BG_bits = pp.BG_bits; d.digitG = pp.digitG; d.Br = pp.Br; d.digitR = pp.digitR;
    d.Bks = pp.Bks; d.digitKS = pp.digitKS; d.Bks_R_bits = pp.Bks_R_bits; d.digitKS_R = pp.digitKS_R;
    for (int i = 0; i < 6; i++) d.gate_constant[i] = pp.gate_constant[i];
    d.gate_constant[6] = d.gate_constant[7] = 0;
    d.mu64 = (uint64_t)(((unsigned __int128)1 << 64) / pp.Q);
    d.ks_row = (uint32_t)(((pp.n + 1) + 31) / 32 * 32);
    if (!wide) {
        d.key_factor = (uint32_t)host::mulmod(((uint64_t)1 << 32) % pp.Q, pp.iN, pp.Q);
        uint32_t inv = 1;   // Q^-1 mod 2^32 by Newton iteration (Q odd)
        for (int it = 0; it < 5; it++) inv *= 2u - (uint32_t)pp.Q * inv;
        d.qinv_neg = 0u - inv;
    }
    d.last_digit_from_acc = pp.BG_bits * pp.digitG >= 64 || (pp.Q >> (pp.BG_bits * pp.digitG)) == 0;
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        g_create_error = std::string("stream creation failed: ") + cudaGetErrorString(e);
        delete c;
        return FHEACC_EIO;
    }
    e = cudaEventCreateWithFlags(&c->done, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        g_create_error = std::string("event creation failed: ") + cudaGetErrorString(e);
        cudaStreamDestroy(c->stream);
        delete c;
        return FHEACC_EIO;
    }
    for (int i = 0; i < 3 && e == cudaSuccess; i++) e = cudaEventCreate(&c->prof[i]);
    if (e != cudaSuccess) {
        g_create_error = std::string("event creation failed: ") + cudaGetErrorString(e);
        fheacc_destroy(reinterpret_cast<fheacc_ctx *>(c));
        return FHEACC_EIO;
    }
    e = cudaMalloc(&c->d_window, (kWindowCapacity + 2) * sizeof(unsigned));
    if (e == cudaSuccess) {
        c->d_status = c->d_window + kWindowCapacity + 1;
        e = cudaMemset(c->d_status, 0, sizeof(unsigned));
    }
    if (e != cudaSuccess) {
        g_create_error = std::string("step-window counters: ") + cudaGetErrorString(e);
        fheacc_destroy(reinterpret_cast<fheacc_ctx *>(c));
        return FHEACC_ENOMEM;
    }
    int rc = build_tables(*c);
    if (rc == FHEACC_OK) rc = build_rotations(*c);
    if (rc != FHEACC_OK) {
        g_create_error = c->err;
        fheacc_destroy(reinterpret_cast<fheacc_ctx *>(c));
        return rc;
    }
    *out = reinterpret_cast<fheacc_ctx *>(c);
    return FHEACC_OK;
}

int fheacc_destroy(fheacc_ctx *ctx)
{
    if (!ctx) return FHEACC_OK;
    Context *c = reinterpret_cast<Context *>(ctx);
    DeviceGuard g(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    cudaFree(c->d_fwd_tw);
    cudaFree(c->d_inv_tw);
    cudaFree(c->d_tw64);
    cudaFree(c->d_itw64);
    cudaFree(c->d_btkey64);
    cudaFree(c->d_cf64);
    cudaFree(c->d_kskey64);
    cudaFree(c->d_subs64);
    cudaFree(c->d_rot);
    cudaFree(c->d_rot_fwd);
    cudaFree(c->d_btkey);
    cudaFree(c->d_kskey);
    cudaFree(c->d_subs);
    cudaFree(c->accs.ptr);
    cudaFree(c->extract.ptr);
    cudaFree(c->io.ptr);
    cudaFree(c->psi.ptr);
    cudaFree(c->expand.ptr);
    cudaFree(c->d_window);
    if (c->done) cudaEventDestroy(c->done);
    for (auto &ev : c->prof)
        if (ev) cudaEventDestroy(ev);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return FHEACC_OK;
}

const char *fheacc_last_error(const fheacc_ctx *ctx)
{
    if (!ctx) return g_create_error.c_str();
    return reinterpret_cast<const Context *>(ctx)->err.c_str();
}

int fheacc_get_params(const fheacc_ctx *ctx, fheacc_params *out)
{
    if (!ctx || !out) return FHEACC_EINVAL;
    *out = reinterpret_cast<const Context *>(ctx)->p;
    return FHEACC_OK;
}

size_t fheacc_device_bytes(const fheacc_ctx *ctx)
{
    return ctx ? reinterpret_cast<const Context *>(ctx)->device_bytes() : 0;
}

// One pass over the bootstrap key in device order, one step (all residues) per
// chunk: upload (verify = false), or compare each chunk as the upload would
// make it with the resident copy (verify = true; FHEACC_EMISMATCH at the first
// chunk that differs).
static int bootstrap_key_pass(Context &c, const uint64_t *btkey, size_t words, bool verify)
{
    const size_t n = c.p.n, dR = c.p.digitR, Br = c.p.Br;
    const size_t rw = (size_t)c.p.digitG * 4 * c.p.N;
    const uint64_t Q = c.p.Q;
    if (verify && !(c.wide ? (void *)c.d_btkey64 : (void *)c.d_btkey))
        return c.fail(FHEACC_ENOKEY, "bootstrap key not uploaded");
    if (c.wide) {
        // device order, one step (all residues) per chunk, Shoup pairs made on the GPU
        if (!verify && !c.d_btkey64) {
            cudaError_t e = cudaMalloc(&c.d_btkey64, words * sizeof(ulonglong2));
            if (e != cudaSuccess) {
                cudaGetLastError();
                c.d_btkey64 = nullptr;
                return c.fail(FHEACC_ENOMEM, "device memory for the bootstrap key");
            }
            c.btkey_bytes = words * sizeof(ulonglong2);
        }
        std::vector<uint64_t> stage(Br * rw);
        uint64_t *d_stage = nullptr;
        ulonglong2 *d_check = nullptr;   // verify: the chunk as the upload makes it
        std::vector<ulonglong2> made, held;
        cudaError_t e = cudaMalloc(&d_stage, Br * rw * sizeof(uint64_t));
        if (e == cudaSuccess && verify) {
            e = cudaMalloc(&d_check, Br * rw * sizeof(ulonglong2));
            made.resize(Br * rw);
            held.resize(Br * rw);
        }
        if (e != cudaSuccess) {
            cudaFree(d_stage);
            return c.cuda_fail(e, "key staging");
        }
        int rc = FHEACC_OK;
        const bool derive = c.dp.last_digit_from_acc != 0;
        for (size_t i = 0; i < n && !rc; i++) {
            for (size_t j = 0; j < dR && !rc; j++) {
                for (size_t r = 0; r < Br; r++)
                    std::memcpy(stage.data() + r * rw, btkey + ((r * dR + j) * n + i) * rw, rw * sizeof(uint64_t));
                e = cudaMemcpy(d_stage, stage.data(), Br * rw * sizeof(uint64_t), cudaMemcpyHostToDevice);
                if (e != cudaSuccess) rc = c.cuda_fail(e, "key upload");
                else if (derive) rc = launch_derive_keys64(c, d_stage, Br, c.d_cf64, c.stream);
                ulonglong2 *chunk = c.d_btkey64 + (i * dR + j) * Br * rw;
                if (!rc) rc = launch_shoup_pairs64(c, d_stage, verify ? d_check : chunk, Br * rw, c.stream);
                if (!rc && cudaStreamSynchronize(c.stream) != cudaSuccess) rc = c.cuda_fail(cudaGetLastError(), "key pairs");
                if (!rc && verify) {
                    e = cudaMemcpy(made.data(), d_check, Br * rw * sizeof(ulonglong2), cudaMemcpyDeviceToHost);
                    if (e == cudaSuccess) e = cudaMemcpy(held.data(), chunk, Br * rw * sizeof(ulonglong2), cudaMemcpyDeviceToHost);
                    if (e != cudaSuccess) rc = c.cuda_fail(e, "key read-back");
                    else if (std::memcmp(made.data(), held.data(), Br * rw * sizeof(ulonglong2)) != 0)
                        rc = c.fail(FHEACC_EMISMATCH, "device bootstrap key differs from the given key");
                }
            }
        }
        cudaFree(d_stage);
        cudaFree(d_check);
        return rc;
    }
    if (!verify && !c.d_btkey) {
        cudaError_t e = cudaMalloc(&c.d_btkey, words * sizeof(uint32_t));
        if (e != cudaSuccess) {
            cudaGetLastError();
            c.d_btkey = nullptr;
            return c.fail(FHEACC_ENOMEM, "device memory for the bootstrap key");
        }
        c.btkey_bytes = words * sizeof(uint32_t);
    }
    // host [r][j][i] -> device [(i * digitR + j) * Br + r], one step (all r) per
    // chunk; words times 2^32 N^-1 mod Q (see DevParams::key_factor)
    const uint64_t kf = c.dp.key_factor, kfs = shoup32_companion(kf, Q);
    // row factors of the last-digit identity (DevParams::last_digit_from_acc):
    // cf[h] = BG^(h - digitG + 1) for h < digitG - 1, cf[digitG - 1] =
    // BG^-(digitG - 1) N. The accumulator it multiplies is stored times N^-1
    // (as all are), so that row must not carry the key factor's N^-1.
    const uint64_t dG = c.p.digitG, plane = 4 * (size_t)c.p.N;   // one row h: [g][P][N]
    std::vector<uint64_t> cf(dG, 1);
    const uint64_t bg_inv = host::powmod(((uint64_t)1 << c.p.BG_bits) % Q, Q - 2, Q);
    for (uint64_t h = 0; h + 1 < dG; h++) cf[h] = host::powmod(bg_inv, dG - 1 - h, Q);
    cf[dG - 1] = host::mulmod(host::powmod(bg_inv, dG - 1, Q), (uint64_t)c.p.N % Q, Q);
    std::vector<uint64_t> cfs(dG);   // Shoup companions: a * cf mod Q for a < Q < 2^32
    for (uint64_t h = 0; h < dG; h++) cfs[h] = shoup32_companion(cf[h], Q);
    auto mulc = [&](uint64_t a, uint64_t h) {
        const uint64_t v = a * cf[h] - ((a * cfs[h]) >> 32) * Q;
        return v >= Q ? v - Q : v;
    };
    const bool derive = c.dp.last_digit_from_acc != 0;
    std::vector<uint32_t> stage(Br * rw), held(verify ? Br * rw : 0);
    std::vector<uint64_t> row(rw);
    for (size_t i = 0; i < n; i++) {
        for (size_t j = 0; j < dR; j++) {
            for (size_t r = 0; r < Br; r++) {
                const uint64_t *src = btkey + ((r * dR + j) * n + i) * rw;
                uint32_t *dst = stage.data() + r * rw;
                for (size_t x = 0; x < rw; x++) row[x] = src[x] % Q;
                if (derive) {
                    const uint64_t *last = row.data() + (dG - 1) * plane;
                    for (uint64_t h = 0; h + 1 < dG; h++)
                        for (size_t x = 0; x < plane; x++)
                            row[h * plane + x] = host::submod(row[h * plane + x], mulc(last[x], h), Q);
                    for (size_t x = 0; x < plane; x++)
                        row[(dG - 1) * plane + x] = mulc(row[(dG - 1) * plane + x], dG - 1);
                }
                for (size_t x = 0; x < rw; x++) {
                    const uint64_t a = row[x];
                    uint64_t v = a * kf - ((a * kfs) >> 32) * Q;   // Shoup: [0, 2Q)
                    dst[(x & ~(size_t)1023) + btile_index(x & 1023)] = (uint32_t)(v >= Q ? v - Q : v);
                }
            }
            uint32_t *chunk = c.d_btkey + (i * dR + j) * Br * rw;
            if (verify) {
                cudaError_t e = cudaMemcpy(held.data(), chunk, Br * rw * sizeof(uint32_t), cudaMemcpyDeviceToHost);
                if (e != cudaSuccess) return c.cuda_fail(e, "key read-back");
                if (std::memcmp(held.data(), stage.data(), Br * rw * sizeof(uint32_t)) != 0)
                    return c.fail(FHEACC_EMISMATCH, "device bootstrap key differs from the given key");
                continue;
            }
            int rc = upload_u32(c, chunk, stage.data(), Br * rw);
            if (rc) return rc;
        }
    }
    return FHEACC_OK;
}

int fheacc_upload_bootstrap_key(fheacc_ctx *ctx, const uint64_t *btkey, size_t words)
{
    if (!ctx) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    if (!btkey || words != fheacc_bootstrap_key_words(&c.p)) return c.fail(FHEACC_EINVAL, "bootstrap key size mismatch");
    DeviceGuard g(c.device);
    return bootstrap_key_pass(c, btkey, words, false);
}

int fheacc_verify_bootstrap_key(fheacc_ctx *ctx, const uint64_t *btkey, size_t words)
{
    if (!ctx) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    if (!btkey || words != fheacc_bootstrap_key_words(&c.p)) return c.fail(FHEACC_EINVAL, "bootstrap key size mismatch");
    DeviceGuard g(c.device);
    return bootstrap_key_pass(c, btkey, words, true);
}

int fheacc_upload_lwe_ks_key(fheacc_ctx *ctx, const uint64_t *kskey, size_t words)
{
    if (!ctx) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    if (!kskey || words != fheacc_lwe_ks_key_words(&c.p)) return c.fail(FHEACC_EINVAL, "LWE key-switch key size mismatch");
    DeviceGuard g(c.device);
    const size_t rows = (size_t)c.p.Bks * c.p.digitKS * c.p.N, w = (size_t)c.p.n + 1, rs = c.dp.ks_row;
    if (c.wide) {
        if (!c.d_kskey64) {
            cudaError_t e = cudaMalloc(&c.d_kskey64, rows * rs * sizeof(uint64_t));
            if (e != cudaSuccess) {
                cudaGetLastError();
                c.d_kskey64 = nullptr;
                return c.fail(FHEACC_ENOMEM, "device memory for the LWE key-switch key");
            }
            c.kskey_bytes = rows * rs * sizeof(uint64_t);
        }
        const size_t chunk = 8192;
        std::vector<uint64_t> stage(chunk * rs, 0);
        for (size_t r0 = 0; r0 < rows; r0 += chunk) {
            const size_t m = std::min(chunk, rows - r0);
            for (size_t r = 0; r < m; r++)
                for (size_t k = 0; k < w; k++) stage[r * rs + k] = kskey[(r0 + r) * w + k] % c.p.Q;
            cudaError_t e = cudaMemcpy(c.d_kskey64 + r0 * rs, stage.data(), m * rs * sizeof(uint64_t),
                                       cudaMemcpyHostToDevice);
            if (e != cudaSuccess) return c.cuda_fail(e, "key upload");
        }
        return FHEACC_OK;
    }
    if (!c.d_kskey) {
        cudaError_t e = cudaMalloc(&c.d_kskey, rows * rs * sizeof(uint32_t));
        if (e != cudaSuccess) {
            cudaGetLastError();
            c.d_kskey = nullptr;
            return c.fail(FHEACC_ENOMEM, "device memory for the LWE key-switch key");
        }
        c.kskey_bytes = rows * rs * sizeof(uint32_t);
    }
    const size_t chunk = 8192;
    std::vector<uint32_t> stage(chunk * rs, 0);
    for (size_t r0 = 0; r0 < rows; r0 += chunk) {
        const size_t m = std::min(chunk, rows - r0);
        for (size_t r = 0; r < m; r++)
            for (size_t k = 0; k < w; k++) stage[r * rs + k] = (uint32_t)(kskey[(r0 + r) * w + k] % c.p.Q);
        int rc = upload_u32(c, c.d_kskey + r0 * rs, stage.data(), m * rs);
        if (rc) return rc;
    }
    return FHEACC_OK;
}

// Upload of the substitute key (verify = false), or comparison of the words the
// upload would make with the resident copy (verify = true; FHEACC_EMISMATCH if
// they differ).
static int subs_key_pass(Context &c, const uint64_t *subs_key, size_t words, bool verify)
{
    if (verify && !(c.wide ? (void *)c.d_subs64 : (void *)c.d_subs))
        return c.fail(FHEACC_ENOKEY, "substitute key not uploaded");
    if (c.wide) {
        if (!verify && !c.d_subs64) {
            cudaError_t e = cudaMalloc(&c.d_subs64, words * sizeof(ulonglong2));
            if (e != cudaSuccess) {
                cudaGetLastError();
                c.d_subs64 = nullptr;
                return c.fail(FHEACC_ENOMEM, "device memory for the substitute key");
            }
            c.subs_bytes = words * sizeof(ulonglong2);
        }
        uint64_t *d_stage = nullptr;
        ulonglong2 *d_check = nullptr;   // verify: the pairs as the upload makes them
        cudaError_t e = cudaMalloc(&d_stage, words * sizeof(uint64_t));
        if (e == cudaSuccess && verify) e = cudaMalloc(&d_check, words * sizeof(ulonglong2));
        if (e == cudaSuccess) e = cudaMemcpy(d_stage, subs_key, words * sizeof(uint64_t), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(d_stage);
            cudaFree(d_check);
            return c.cuda_fail(e, "substitute key upload");
        }
        int rc = launch_shoup_pairs64(c, d_stage, verify ? d_check : c.d_subs64, words, c.stream);
        if (!rc && cudaStreamSynchronize(c.stream) != cudaSuccess) rc = c.cuda_fail(cudaGetLastError(), "key pairs");
        if (!rc && verify) {
            std::vector<ulonglong2> made(words), held(words);
            e = cudaMemcpy(made.data(), d_check, words * sizeof(ulonglong2), cudaMemcpyDeviceToHost);
            if (e == cudaSuccess) e = cudaMemcpy(held.data(), c.d_subs64, words * sizeof(ulonglong2), cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) rc = c.cuda_fail(e, "key read-back");
            else if (std::memcmp(made.data(), held.data(), words * sizeof(ulonglong2)) != 0)
                rc = c.fail(FHEACC_EMISMATCH, "device substitute key differs from the given key");
        }
        cudaFree(d_stage);
        cudaFree(d_check);
        return rc;
    }
    if (!verify && !c.d_subs) {
        cudaError_t e = cudaMalloc(&c.d_subs, words * sizeof(uint32_t));
        if (e != cudaSuccess) {
            cudaGetLastError();
            c.d_subs = nullptr;
            return c.fail(FHEACC_ENOMEM, "device memory for the substitute key");
        }
        c.subs_bytes = words * sizeof(uint32_t);
    }
    std::vector<uint32_t> stage(words);
    for (size_t x = 0; x < words; x++) stage[x] = (uint32_t)(subs_key[x] % c.p.Q);
    if (!verify) return upload_u32(c, c.d_subs, stage.data(), words);
    std::vector<uint32_t> held(words);
    cudaError_t e = cudaMemcpy(held.data(), c.d_subs, words * sizeof(uint32_t), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return c.cuda_fail(e, "key read-back");
    return std::memcmp(held.data(), stage.data(), words * sizeof(uint32_t)) == 0
               ? FHEACC_OK
               : c.fail(FHEACC_EMISMATCH, "device substitute key differs from the given key");
}

int fheacc_upload_subs_key(fheacc_ctx *ctx, const uint64_t *subs_key, size_t words)
{
    if (!ctx) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    if (!subs_key || words != fheacc_subs_key_words(&c.p)) return c.fail(FHEACC_EINVAL, "substitute key size mismatch");
    DeviceGuard g(c.device);
    return subs_key_pass(c, subs_key, words, false);
}

int fheacc_verify_subs_key(fheacc_ctx *ctx, const uint64_t *subs_key, size_t words)
{
    if (!ctx) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    if (!subs_key || words != fheacc_subs_key_words(&c.p)) return c.fail(FHEACC_EINVAL, "substitute key size mismatch");
    DeviceGuard g(c.device);
    return subs_key_pass(c, subs_key, words, true);
}

int fheacc_bootstrap_async(fheacc_ctx *ctx, const uint64_t *d_c1, const uint64_t *d_c2, const int32_t *d_gates,
                           size_t count, uint64_t *d_out, uint32_t flags, void *stream)
{
    if (!ctx) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    if (count && (!d_c1 || !d_c2 || !d_gates || !d_out)) return c.fail(FHEACC_EINVAL, "null buffer");
    DeviceGuard g(c.device);
    cudaStream_t st = pick_stream(&c, stream);
    return mark_done(c, st, bootstrap_device(c, d_c1, d_c2, d_gates, count, d_out, flags, st, 0));
}

int fheacc_bootstrap_plain_async(fheacc_ctx *ctx, const uint64_t *d_c1, const uint64_t *d_c2,
                                 const int32_t *d_gates, size_t count, uint64_t *d_out, uint32_t flags,
                                 void *stream)
{
    if (!ctx) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    if (count && (!d_c1 || !d_c2 || !d_gates || !d_out)) return c.fail(FHEACC_EINVAL, "null buffer");
    DeviceGuard g(c.device);
    cudaStream_t st = pick_stream(&c, stream);
    const size_t w = (size_t)c.p.n + 1;
    for (size_t i = 0; i < count; i++) {
        int rc = bootstrap_device(c, d_c1 + i * w, d_c2 + i * w, d_gates + i, 1, d_out + i * w, flags, st, 1);
        if (rc) return rc;
    }
    return mark_done(c, st, FHEACC_OK);
}

int fheacc_bootstrap(fheacc_ctx *ctx, const uint64_t *c1, const uint64_t *c2, const int32_t *gates, size_t count,
                     uint64_t *out, uint32_t flags)
{
    if (!ctx) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    if (count == 0) return FHEACC_OK;
    if (!c1 || !c2 || !gates || !out) return c.fail(FHEACC_EINVAL, "null buffer");
    const size_t w = (size_t)c.p.n + 1;
    for (size_t i = 0; i < count; i++) {
        if (gates[i] < 0 || gates[i] > 5) return c.fail(FHEACC_EINVAL, "gate code out of range");
        if (std::memcmp(c1 + i * w, c2 + i * w, w * sizeof(uint64_t)) == 0)
            return c.fail(FHEACC_EINVAL, "c1 == c2: only independent ciphertexts can be bootstrapped");
    }
    DeviceGuard g(c.device);
    const size_t lwe_bytes = count * w * sizeof(uint64_t);
    const size_t gate_off = (3 * lwe_bytes + 255) / 256 * 256;
    int rc = ensure_scratch(c, c.io, gate_off + count * sizeof(int32_t));
    if (rc) return rc;
    char *base = (char *)c.io.ptr;
    uint64_t *d_c1 = (uint64_t *)base, *d_c2 = (uint64_t *)(base + lwe_bytes), *d_out = (uint64_t *)(base + 2 * lwe_bytes);
    int32_t *d_g = (int32_t *)(base + gate_off);
    cudaStream_t st = c.stream;
    cudaError_t e = cudaMemcpyAsync(d_c1, c1, lwe_bytes, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_c2, c2, lwe_bytes, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_g, gates, count * sizeof(int32_t), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return c.cuda_fail(e, "input copy");
    rc = bootstrap_device(c, d_c1, d_c2, d_g, count, d_out, flags, st, 0);
    if (rc) return rc;
    e = cudaMemcpyAsync(out, d_out, lwe_bytes, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return c.cuda_fail(e, "bootstrap");
    return take_device_status(c, nullptr);
}

int fheacc_ntt_forward(fheacc_ctx *ctx, uint64_t *d_polys, size_t count, void *stream)
{
    if (!ctx) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    DeviceGuard g(c.device);
    cudaStream_t st = pick_stream(&c, stream);
    return mark_done(c, st, c.wide ? launch_ntt64(c, d_polys, count, false, st) : launch_ntt32(c, d_polys, count, false, st));
}

int fheacc_ntt_inverse(fheacc_ctx *ctx, uint64_t *d_polys, size_t count, void *stream)
{
    if (!ctx) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    DeviceGuard g(c.device);
    cudaStream_t st = pick_stream(&c, stream);
    return mark_done(c, st, c.wide ? launch_ntt64(c, d_polys, count, true, st) : launch_ntt32(c, d_polys, count, true, st));
}

int fheacc_rlwe_mult_rgsw(fheacc_ctx *ctx, const uint64_t *d_acc, const uint64_t *d_rgsw, uint64_t *d_out,
                          size_t count, void *stream)
{
    if (!ctx) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    DeviceGuard g(c.device);
    cudaStream_t st = pick_stream(&c, stream);
    const size_t stride = (size_t)c.p.digitG * 4 * c.p.N;
    return mark_done(c, st, c.wide ? launch_rlwe_mult_rgsw64(c, d_acc, d_rgsw, d_out, count, stride, st)
                                   : launch_rlwe_mult_rgsw32(c, d_acc, d_rgsw, d_out, count, stride, st));
}

int fheacc_blind_rotate_async(fheacc_ctx *ctx, const uint64_t *d_c1, const uint64_t *d_c2, const int32_t *d_gates,
                              size_t count, uint64_t *d_acc, uint32_t flags, void *stream)
{
    if (!ctx) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    DeviceGuard g(c.device);
    cudaStream_t st = pick_stream(&c, stream);
    if (c.wide) return mark_done(c, st, launch_blind_rotate64(c, d_c1, d_c2, d_gates, count, flags, d_acc, nullptr, 0, st));
    return mark_done(c, st, launch_blind_rotate32(c, d_c1, d_c2, d_gates, count, flags, d_acc, nullptr, 0, st));
}

int fheacc_lwe_keyswitch_async(fheacc_ctx *ctx, const uint64_t *d_rlwe, size_t count, uint64_t *d_out,
                               void *stream)
{
    if (!ctx) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    DeviceGuard g(c.device);
    cudaStream_t st = pick_stream(&c, stream);
    if (c.wide) {
        int rc = ensure_scratch(c, c.extract, count * kExtract64 * sizeof(uint64_t));
        if (rc) return rc;
        rc = launch_extract64(c, d_rlwe, count, (uint64_t *)c.extract.ptr, st);
        if (rc) return rc;
        return mark_done(c, st, launch_lwe_keyswitch64(c, (uint64_t *)c.extract.ptr, count, false, d_out, st));
    }
    int rc = ensure_scratch(c, c.extract, count * kExtractStride * sizeof(uint32_t));
    if (rc) return rc;
    rc = launch_extract_from_ntt32(c, d_rlwe, count, (uint32_t *)c.extract.ptr, st);
    if (rc) return rc;
    return mark_done(c, st, launch_lwe_keyswitch32(c, (uint32_t *)c.extract.ptr, count, false, d_out, st));
}

int fheacc_lwe_modswitch_async(fheacc_ctx *ctx, const uint64_t *d_in, size_t count, uint64_t *d_out, void *stream)
{
    if (!ctx) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    DeviceGuard g(c.device);
    cudaStream_t st = pick_stream(&c, stream);
    return mark_done(c, st, launch_modswitch(c, d_in, count, d_out, st));
}

int fheacc_set_option(fheacc_ctx *ctx, int option, int value)
{
    if (!ctx) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    switch (option) {
    case FHEACC_OPT_BR_REGS_FOR_3:
        c.tune.br_regs_for_3 = value < 0 ? -1 : value ? 1 : 0;
        return FHEACC_OK;
    case FHEACC_OPT_BR_CTAS_PER_SM:
        if (value < 0 || value > 32) return c.fail(FHEACC_EINVAL, "CTAs per SM out of range");
        c.tune.br_ctas_per_sm = value;
        return FHEACC_OK;
    case FHEACC_OPT_BR_GROUP:
        if (value < 0 || value > 64) return c.fail(FHEACC_EINVAL, "group size out of range");
        c.tune.br_group = value;
        return FHEACC_OK;
    case FHEACC_OPT_BR_PIPES:
        if (value < 0 || value > 3) return c.fail(FHEACC_EINVAL, "pipelines per CTA must be 0..3");
        c.tune.br_pipes = value;
        return FHEACC_OK;
    case FHEACC_OPT_BR_WINDOW:
        if (value < -1 || value > 1024) return c.fail(FHEACC_EINVAL, "step window out of range");
        c.tune.br_window = value;
        return FHEACC_OK;
    case FHEACC_OPT_BR_POOL:
        c.tune.br_pool = value < 0 ? -1 : value ? 1 : 0;
        return FHEACC_OK;
    case FHEACC_OPT_KS_TILED:
        c.tune.ks_tiled = value < 0 ? -1 : value ? 1 : 0;
        return FHEACC_OK;
    case FHEACC_OPT_BR_SOLO:
        if (value < -1 || value > 64) return c.fail(FHEACC_EINVAL, "latency-form gates per SM must be -1..64");
        c.tune.br_solo = value;
        return FHEACC_OK;
    case FHEACC_OPT_DEBUG_WAIT_LIMIT:
        if (value < -1) return c.fail(FHEACC_EINVAL, "wait limit must be -1 (built-in) or >= 0");
        c.tune.debug_wait_limit = value;
        return FHEACC_OK;

    default:
        return c.fail(FHEACC_EINVAL, "unknown option");
    }
}

int fheacc_kernel_times(fheacc_ctx *ctx, float ms[2])
{
    if (!ctx || !ms) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    DeviceGuard g(c.device);
    cudaError_t e = cudaEventSynchronize(c.prof[2]);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms[0], c.prof[0], c.prof[1]);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms[1], c.prof[1], c.prof[2]);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return c.cuda_fail(e, "kernel times (no profiled call yet?)");
    }
    return FHEACC_OK;
}

int fheacc_measure_imad_rate(fheacc_ctx *ctx, double *imad_per_s)
{
    if (!ctx || !imad_per_s) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    DeviceGuard g(c.device);
    return measure_imad_rate(c, imad_per_s);
}

int fheacc_measure_l2_read_rate(fheacc_ctx *ctx, double *bytes_per_s)
{
    if (!ctx || !bytes_per_s) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    DeviceGuard g(c.device);
    return measure_l2_read_rate(c, bytes_per_s);
}

int fheacc_measure_components(fheacc_ctx *ctx, double ns[4])
{
    if (!ctx || !ns) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    DeviceGuard g(c.device);
    return measure_components(c, ns);
}

static const void *subs_key_level(Context &c, int f)
{
    const size_t per = (size_t)c.p.digitKS_R * 2 * c.p.N;
    if (c.wide) return c.d_subs64 ? (const void *)(c.d_subs64 + (size_t)f * per) : nullptr;
    return c.d_subs ? (const void *)(c.d_subs + (size_t)f * per) : nullptr;
}

int fheacc_rlwe_substitute_async(fheacc_ctx *ctx, const uint64_t *d_in, size_t count, int f, uint64_t *d_out,
                                 void *stream)
{
    if (!ctx) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    DeviceGuard g(c.device);
    cudaStream_t st = pick_stream(&c, stream);
    return mark_done(c, st, launch_expand(c, 0, d_in, d_out, count, f, nullptr, nullptr, st));
}

int fheacc_rlwe_keyswitch_async(fheacc_ctx *ctx, const uint64_t *d_in, size_t count, const uint64_t *d_ksk,
                                uint64_t *d_out, void *stream)
{
    if (!ctx) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    if (count && !d_ksk) return c.fail(FHEACC_EINVAL, "null key");
    DeviceGuard g(c.device);
    cudaStream_t st = pick_stream(&c, stream);
    const size_t words = (size_t)c.p.digitKS_R * 2 * c.p.N;
    int rc = ensure_scratch(c, c.io, words * (c.wide ? sizeof(ulonglong2) : sizeof(uint32_t)));
    if (rc) return rc;
    rc = c.wide ? launch_shoup_pairs64(c, d_ksk, (ulonglong2 *)c.io.ptr, words, st)
                : launch_to_u32(c, d_ksk, (uint32_t *)c.io.ptr, words, st);
    if (rc) return rc;
    return mark_done(c, st, launch_expand(c, 1, d_in, d_out, count, 0, c.io.ptr, nullptr, st));
}

int fheacc_subs_keyswitch_async(fheacc_ctx *ctx, const uint64_t *d_in, size_t count, int f, uint64_t *d_out,
                                void *stream)
{
    if (!ctx) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    const int logN = c.wide ? 11 : 10;
    if (f < 0 || f >= logN) return c.fail(FHEACC_EINVAL, "substitution factor out of range");
    const void *key = subs_key_level(c, f);
    if (!key) return c.fail(FHEACC_ENOKEY, "substitute key not uploaded");
    DeviceGuard g(c.device);
    cudaStream_t st = pick_stream(&c, stream);
    return mark_done(c, st, launch_expand(c, 2, d_in, d_out, count, f, key, nullptr, st));
}

}  // extern "C"

namespace fheacc {

int expand_device(Context &c, const uint64_t *d_in, uint64_t *d_out, cudaStream_t st, size_t count)
{
    if (!subs_key_level(c, 0)) return c.fail(FHEACC_ENOKEY, "substitute key not uploaded");
    if (!count) return FHEACC_OK;
    const int N = c.p.N, logN = c.wide ? 11 : 10;
    const size_t rw = 2 * (size_t)N, stride = (size_t)N * rw;   // one RLWE; one expansion's output
    // r[0] of every expansion = its input
    cudaError_t e = cudaMemcpy2DAsync(d_out, stride * sizeof(uint64_t), d_in, rw * sizeof(uint64_t),
                                      rw * sizeof(uint64_t), count, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return c.cuda_fail(e, "expand copy");
    for (int f = 0; f < logN; f++) {
        int rc = launch_expand(c, 3, d_out, d_out, 0, f, subs_key_level(c, f), c.d_rot + (size_t)f * N, st, count,
                               stride);
        if (rc) return rc;
    }
    return FHEACC_OK;
}

}  // namespace fheacc

extern "C" {

int fheacc_expand_rlwe(fheacc_ctx *ctx, const uint64_t *d_in, uint64_t *d_out, void *stream)
{
    if (!ctx) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    if (!d_in || !d_out) return c.fail(FHEACC_EINVAL, "null buffer");
    DeviceGuard g(c.device);
    cudaStream_t st = pick_stream(&c, stream);
    return mark_done(c, st, expand_device(c, d_in, d_out, st));
}

int fheacc_device_status(fheacc_ctx *ctx, uint32_t *bits)
{
    if (!ctx) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    DeviceGuard g(c.device);
    return take_device_status(c, bits);
}

int fheacc_kernel_launches(const fheacc_ctx *ctx, uint64_t *count)
{
    if (!ctx || !count) return FHEACC_EINVAL;
    *count = reinterpret_cast<const Context *>(ctx)->launches.load(std::memory_order_relaxed);
    return FHEACC_OK;
}

int fheacc_sync(fheacc_ctx *ctx, uint32_t timeout_ms)
{
    if (!ctx) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    DeviceGuard g(c.device);
    auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        cudaError_t e = cudaStreamQuery(c.stream);
        if (e == cudaSuccess) e = cudaEventQuery(c.done);
        if (e == cudaSuccess) return take_device_status(c, nullptr);
        if (e != cudaErrorNotReady) return c.cuda_fail(e, "sync");
        if (timeout_ms) {
            auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count();
            if (ms >= (long long)timeout_ms) return c.fail(FHEACC_ETIMEDOUT, "sync timed out");
        }
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
}

}  // extern "C"
