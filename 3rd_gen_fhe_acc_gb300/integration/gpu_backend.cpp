// gpu_backend.cpp -- namespace GPU over libfheacc.so; see gpu_backend.h.
//
// Each call flattens the runtime's objects into the word layouts of
// include/fheacc.h (the reference's own std::vector orders), calls the C ABI
// and rebuilds the runtime's objects from the result. The reference runtime's
// globals (params.h) describe the parameter set, as they do for the FPGA
// backend (OCL_config_wr_rd pushes them to the card, myfpga.cpp:82-326).
#include "gpu_backend.h"

#include <cerrno>
#include <cstring>
#include <cuda_runtime.h>

namespace GPU {
namespace {

constexpr int kSlots = 16;

struct Slot {
    fheacc_ctx *ctx = nullptr;
    const RLWE::bootstrap_key *bt = nullptr;  // eval_bootstrap's key object on the device (nullptr: uploaded by dma_write)
    const LWE::keyswitch_key *ks = nullptr;   // the key switch key on the device
    uint64_t *d_enc_sec = nullptr;            // RGSW(-s) of dma_write_RGSW_enc_sk
    bool subs = false;
};

Slot g_slot[kSlots];
uint32_t g_flags = 0;

Slot *slot_of(int slot_id)
{
    return slot_id >= 0 && slot_id < kSlots && g_slot[slot_id].ctx ? &g_slot[slot_id] : nullptr;
}

// the FPGA calls' rc: -ENOMEM for a failed allocation, -1 otherwise
int fpga_rc(int code) { return code == FHEACC_OK ? 0 : code == FHEACC_ENOMEM ? -ENOMEM : -1; }

void flat_lwe(const LWE::LWE_ciphertext &c, uint64_t *o)
{
    for (int i = 0; i < n; i++) o[i] = c.a[i];
    o[n] = c.b;
}

LWE::LWE_ciphertext lwe_of(const uint64_t *w)
{
    LWE::LWE_ciphertext c;
    for (int i = 0; i < n; i++) c.a[i] = w[i];
    c.b = w[n];
    return c;
}

void flat_rlwe(const RLWE::RLWE_ciphertext &c, uint64_t *o)
{
    for (int i = 0; i < N; i++) {
        o[i] = c.a[i];
        o[N + i] = c.b[i];
    }
}

RLWE::RLWE_ciphertext rlwe_of(const uint64_t *w)
{
    RLWE::RLWE_ciphertext c;
    for (int i = 0; i < N; i++) {
        c.a[i] = w[i];
        c.b[i] = w[N + i];
    }
    c.NTT_form = true;
    return c;
}

// RGSW c_text[h][g] -> [digitG][2][2][N]
void flat_rgsw(const RLWE::RGSW_ciphertext &g, uint64_t *o)
{
    for (uint64_t h = 0; h < digitG; h++)
        for (int r = 0; r < 2; r++) flat_rlwe(g.c_text[h][r], o + (h * 2 + r) * 2 * (size_t)N);
}

RLWE::RGSW_ciphertext rgsw_of(const uint64_t *w)
{
    RLWE::RGSW_ciphertext g;
    g.c_text.resize(digitG);
    for (uint64_t h = 0; h < digitG; h++) {
        g.c_text[h].resize(2);
        for (int r = 0; r < 2; r++) g.c_text[h][r] = rlwe_of(w + (h * 2 + r) * 2 * (size_t)N);
    }
    return g;
}

int upload_kskey(Slot &s, const LWE::keyswitch_key &ks)
{
    if (s.ks == &ks) return FHEACC_OK;
    std::vector<uint64_t> w;
    w.reserve((size_t)Bks * digitKS * N * (n + 1));
    for (const auto &d : ks.kskey)
        for (const auto &j : d)
            for (const auto &c : j) {
                w.insert(w.end(), c.a.begin(), c.a.begin() + n);
                w.push_back(c.b);
            }
    int rc = fheacc_upload_lwe_ks_key(s.ctx, w.data(), w.size());
    if (rc == FHEACC_OK) s.ks = &ks;
    return rc;
}

// Bootstraps of `count` gates through the host-buffer entry point.
std::vector<LWE::LWE_ciphertext> bootstrap(const std::vector<LWE::LWE_ciphertext> &c1,
                                           const std::vector<LWE::LWE_ciphertext> &c2,
                                           const LWE::keyswitch_key &kskey, const std::vector<GATES> &gate,
                                           size_t count, int *rc)
{
    std::vector<LWE::LWE_ciphertext> out(count);
    Slot *s = slot_of(0);
    for (int i = 0; !s && i < kSlots; i++) s = slot_of(i);
    if (!s) {
        *rc = -1;
        return out;
    }
    int r = upload_kskey(*s, kskey);
    if (r != FHEACC_OK) {
        *rc = fpga_rc(r);
        return out;
    }
    const size_t w = (size_t)n + 1;
    std::vector<uint64_t> a(count * w), b(count * w), o(count * w);
    std::vector<int32_t> g(count);
    for (size_t i = 0; i < count; i++) {
        flat_lwe(c1[i], &a[i * w]);
        flat_lwe(c2[i], &b[i * w]);
        g[i] = (int32_t)gate[i];
    }
    r = fheacc_bootstrap(s->ctx, a.data(), b.data(), g.data(), count, o.data(), g_flags);
    *rc = fpga_rc(r);
    if (r == FHEACC_OK)
        for (size_t i = 0; i < count; i++) out[i] = lwe_of(&o[i * w]);
    return out;
}

std::vector<LWE::LWE_ciphertext> fixed_width(size_t width, const std::vector<LWE::LWE_ciphertext> &c1,
                                             const std::vector<LWE::LWE_ciphertext> &c2,
                                             const LWE::keyswitch_key &kskey, const std::vector<GATES> &gate,
                                             int *rc)
{
    // the FPGA calls check the sizes of c1 and c2 (myfpga.cpp:1140-1144,
    // 1408-1412, 1540-1544); the gate vector must cover them
    if (c1.size() != width || c2.size() != width || gate.size() < width) {
        *rc = -1;
        return std::vector<LWE::LWE_ciphertext>(width);
    }
    return bootstrap(c1, c2, kskey, gate, width, rc);
}

}  // namespace

int OCL_config_wr_rd(const int slot_id)
{
    if (slot_id < 0 || slot_id >= kSlots) return -1;
    release(slot_id);
    fheacc_params p;
    std::memset(&p, 0, sizeof p);
    p.n = n;
    p.q = (uint32_t)q;
    p.N = N;
    p.Q = Q;
    p.BG_bits = (uint32_t)BGbits;
    p.digitG = (uint32_t)digitG;
    p.Br = (uint32_t)Br;
    p.digitR = (uint32_t)digitR;
    p.Bks = (uint32_t)Bks;
    p.digitKS = (uint32_t)digitKS;
    p.Bks_R_bits = (uint32_t)Bks_R_bits;
    p.digitKS_R = (uint32_t)digitKS_R;
    for (int g = 0; g < 6; g++) p.gate_constant[g] = gate_constant[g];
    p.ROU = ROU;
    p.iN = iN;
    p.E_rlwe = (uint32_t)E_rlwe;
    return fpga_rc(fheacc_create(&p, slot_id, &g_slot[slot_id].ctx));
}

int BAR1_ROU_table_2k_wr(const int slot_id) { return slot_of(slot_id) ? 0 : -1; }
int BAR1_ROU_table_1k_wr(const int slot_id) { return slot_of(slot_id) ? 0 : -1; }

namespace {

// The runtime's key objects as the C ABI's words (btkey[r][j][i].c_text[h][g],
// subs_key[l].RLWE_kskey[k]).
std::vector<uint64_t> flat_bootstrap_key(const RLWE::bootstrap_key &bt_key)
{
    std::vector<uint64_t> w;
    w.reserve((size_t)Br * digitR * n * digitG * 4 * N);
    for (uint64_t r = 0; r < Br; r++)
        for (uint64_t j = 0; j < digitR; j++)
            for (int i = 0; i < n; i++) {
                const size_t at = w.size();
                w.resize(at + (size_t)digitG * 4 * N);
                flat_rgsw(bt_key.btkey[r][j][i], &w[at]);
            }
    return w;
}

std::vector<uint64_t> flat_subs_key(const application::substitute_key &subs_key)
{
    std::vector<uint64_t> w;
    w.reserve((size_t)digitN * digitKS_R * 2 * N);
    for (const auto &level : subs_key.subs_key)
        for (const auto &c : level.RLWE_kskey) {
            const size_t at = w.size();
            w.resize(at + 2 * (size_t)N);
            flat_rlwe(c, &w[at]);
        }
    return w;
}

// a read-back comparison's rc: 0 equal, -ENOMEM, -1 otherwise (a difference included)
int compare_rc(int code) { return code == FHEACC_OK ? 0 : code == FHEACC_ENOMEM ? -ENOMEM : -1; }

}  // namespace

int check_slot_config(int slot_id)
{
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return slot_id >= 0 && slot_id < count && slot_id < kSlots ? 0 : 1;
}

uint64_t buffer_compare(uint8_t *bufa, uint8_t *bufb, size_t buffer_size)
{
    uint64_t differ = 0;
    for (size_t i = 0; i < buffer_size; i++) differ += bufa[i] != bufb[i];
    return differ;
}

int dma_write_bootstrap_key(const int slot_id, const RLWE::bootstrap_key &bt_key)
{
    Slot *s = slot_of(slot_id);
    if (!s) return -1;
    const std::vector<uint64_t> w = flat_bootstrap_key(bt_key);
    s->bt = nullptr;
    return fpga_rc(fheacc_upload_bootstrap_key(s->ctx, w.data(), w.size()));
}

LWE::LWE_ciphertext eval_bootstrap(const LWE::LWE_ciphertext &c1, const LWE::LWE_ciphertext &c2,
                                   const RLWE::bootstrap_key &btkey, const LWE::keyswitch_key &kskey, const GATES gate)
{
    int sid = 0;
    while (sid < kSlots && !slot_of(sid)) sid++;
    if (sid == kSlots) return LWE::LWE_ciphertext();
    Slot *s = slot_of(sid);
    if (s->bt != &btkey) {
        if (dma_write_bootstrap_key(sid, btkey) != 0) return LWE::LWE_ciphertext();
        s->bt = &btkey;
    }
    int rc = 0;
    std::vector<LWE::LWE_ciphertext> out = bootstrap({c1}, {c2}, kskey, {gate}, 1, &rc);
    return rc == 0 ? out[0] : LWE::LWE_ciphertext();
}

int dma_write_subs_key(const int slot_id, const application::substitute_key &subs_key)
{
    Slot *s = slot_of(slot_id);
    if (!s) return -1;
    const std::vector<uint64_t> w = flat_subs_key(subs_key);
    const int r = fheacc_upload_subs_key(s->ctx, w.data(), w.size());
    s->subs = r == FHEACC_OK;
    return fpga_rc(r);
}

int dma_read_compare_bootstrap_key(const int slot_id, const RLWE::bootstrap_key &bt_key)
{
    Slot *s = slot_of(slot_id);
    if (!s) return -1;
    const std::vector<uint64_t> w = flat_bootstrap_key(bt_key);
    return compare_rc(fheacc_verify_bootstrap_key(s->ctx, w.data(), w.size()));
}

int dma_read_compare_subs_key(const int slot_id, const application::substitute_key &subs_key)
{
    Slot *s = slot_of(slot_id);
    if (!s) return -1;
    const std::vector<uint64_t> w = flat_subs_key(subs_key);
    return compare_rc(fheacc_verify_subs_key(s->ctx, w.data(), w.size()));
}

int dma_write_RGSW_enc_sk(const int slot_id, const RLWE::RGSW_ciphertext &enc_sec)
{
    Slot *s = slot_of(slot_id);
    if (!s) return -1;
    const size_t words = (size_t)digitG * 4 * N;
    std::vector<uint64_t> w(words);
    flat_rgsw(enc_sec, w.data());
    int dev = 0;
    cudaGetDevice(&dev);
    cudaSetDevice(slot_id);
    cudaError_t e = cudaSuccess;
    if (!s->d_enc_sec) e = cudaMalloc(&s->d_enc_sec, words * sizeof(uint64_t));
    if (e == cudaSuccess) e = cudaMemcpy(s->d_enc_sec, w.data(), words * sizeof(uint64_t), cudaMemcpyHostToDevice);
    cudaSetDevice(dev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? -ENOMEM : -1;
    }
    return 0;
}

int dma_read_compare_RGSW_enc_sk(const int slot_id, const RLWE::RGSW_ciphertext &enc_sec)
{
    Slot *s = slot_of(slot_id);
    if (!s || !s->d_enc_sec) return -1;
    const size_t words = (size_t)digitG * 4 * N;
    std::vector<uint64_t> want(words), held(words);
    flat_rgsw(enc_sec, want.data());
    int dev = 0;
    cudaGetDevice(&dev);
    cudaSetDevice(slot_id);
    const cudaError_t e = cudaMemcpy(held.data(), s->d_enc_sec, words * sizeof(uint64_t), cudaMemcpyDeviceToHost);
    cudaSetDevice(dev);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    return buffer_compare(reinterpret_cast<uint8_t *>(want.data()), reinterpret_cast<uint8_t *>(held.data()),
                          words * sizeof(uint64_t)) == 0
               ? 0
               : -1;
}

LWE::LWE_ciphertext fpga_eval_bootstrap_x1(const LWE::LWE_ciphertext &c1, const LWE::LWE_ciphertext &c2,
                                           const LWE::keyswitch_key &kskey, const GATES gate,
                                           const pci_bar_handle_t, int *rc, int)
{
    std::vector<LWE::LWE_ciphertext> out = bootstrap({c1}, {c2}, kskey, {gate}, 1, rc);
    return *rc == 0 ? out[0] : LWE::LWE_ciphertext();
}

std::vector<LWE::LWE_ciphertext> fpga_eval_bootstrap_x4(const std::vector<LWE::LWE_ciphertext> &c1,
                                                        const std::vector<LWE::LWE_ciphertext> &c2,
                                                        const LWE::keyswitch_key &kskey,
                                                        const std::vector<GATES> gate, const pci_bar_handle_t,
                                                        int *rc, int)
{
    return fixed_width(4, c1, c2, kskey, gate, rc);
}

std::vector<LWE::LWE_ciphertext> fpga_eval_bootstrap_x8(const std::vector<LWE::LWE_ciphertext> &c1,
                                                        const std::vector<LWE::LWE_ciphertext> &c2,
                                                        const LWE::keyswitch_key &kskey,
                                                        const std::vector<GATES> gate, const pci_bar_handle_t,
                                                        int *rc, int)
{
    return fixed_width(8, c1, c2, kskey, gate, rc);
}

std::vector<LWE::LWE_ciphertext> fpga_eval_bootstrap_x12(const std::vector<LWE::LWE_ciphertext> &c1,
                                                         const std::vector<LWE::LWE_ciphertext> &c2,
                                                         const LWE::keyswitch_key &kskey,
                                                         const std::vector<GATES> gate, const pci_bar_handle_t,
                                                         int *rc, int)
{
    return fixed_width(12, c1, c2, kskey, gate, rc);
}

std::vector<LWE::LWE_ciphertext> fpga_eval_bootstrap_x16(const std::vector<LWE::LWE_ciphertext> &c1,
                                                         const std::vector<LWE::LWE_ciphertext> &c2,
                                                         const LWE::keyswitch_key &kskey,
                                                         const std::vector<GATES> gate, const pci_bar_handle_t,
                                                         int *rc, int)
{
    return fixed_width(10, c1, c2, kskey, gate, rc);
}

namespace {

// A device buffer of `words` u64 for the duration of one call.
struct DevBuf {
    uint64_t *p = nullptr;
    cudaError_t e = cudaSuccess;
    explicit DevBuf(size_t words) { e = cudaMalloc(&p, words * sizeof(uint64_t)); }
    ~DevBuf()
    {
        if (p) cudaFree(p);
    }
};

}  // namespace

std::unique_ptr<std::vector<RLWE::RLWE_ciphertext>> fpga_expand_RLWE(const RLWE::RLWE_ciphertext &c1,
                                                                     const pci_bar_handle_t, int *rc, int, int)
{
    Slot *s = nullptr;
    int sid = 0;
    for (; sid < kSlots && !(s = slot_of(sid)); sid++) {
    }
    if (!s || !s->subs || !c1.NTT_form) {
        *rc = -1;
        return nullptr;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaSetDevice(sid);
    std::unique_ptr<std::vector<RLWE::RLWE_ciphertext>> result;
    {
        const size_t rw = 2 * (size_t)N;
        std::vector<uint64_t> in(rw), out(rw * N);
        flat_rlwe(c1, in.data());
        DevBuf din(rw), dout(rw * N);
        cudaError_t e = din.e != cudaSuccess ? din.e : dout.e;
        if (e == cudaSuccess) e = cudaMemcpy(din.p, in.data(), rw * sizeof(uint64_t), cudaMemcpyHostToDevice);
        int r = e == cudaSuccess ? fheacc_expand_rlwe(s->ctx, din.p, dout.p, nullptr) : FHEACC_EIO;
        if (r == FHEACC_OK) r = fheacc_sync(s->ctx, 0);
        if (r == FHEACC_OK && cudaMemcpy(out.data(), dout.p, out.size() * sizeof(uint64_t),
                                         cudaMemcpyDeviceToHost) != cudaSuccess)
            r = FHEACC_EIO;
        if (e == cudaErrorMemoryAllocation) r = FHEACC_ENOMEM;
        cudaGetLastError();
        *rc = fpga_rc(r);
        if (r == FHEACC_OK) {
            result = std::make_unique<std::vector<RLWE::RLWE_ciphertext>>(N);
            for (int i = 0; i < N; i++) (*result)[i] = rlwe_of(&out[i * rw]);
        }
    }
    cudaSetDevice(dev);
    return result;
}

std::unique_ptr<std::vector<RLWE::RLWE_ciphertext>> fpga_expand_RLWE_cont_rd_wr(const RLWE::RLWE_ciphertext &c1,
                                                                                const pci_bar_handle_t bar, int *rc,
                                                                                int read_fd, int write_fd)
{
    return fpga_expand_RLWE(c1, bar, rc, read_fd, write_fd);
}

std::unique_ptr<std::vector<RLWE::RLWE_ciphertext>> fpga_expand_RLWE_batch_rd_wr(const RLWE::RLWE_ciphertext &c1,
                                                                                 const pci_bar_handle_t bar, int *rc,
                                                                                 int read_fd, int write_fd)
{
    return fpga_expand_RLWE(c1, bar, rc, read_fd, write_fd);
}

std::shared_ptr<std::vector<RLWE::RGSW_ciphertext>> fpga_homo_expand(
    const std::unique_ptr<std::vector<RLWE::RLWE_ciphertext>> &packed_bits, const pci_bar_handle_t, int *rc, int,
    int)
{
    Slot *s = nullptr;
    int sid = 0;
    for (; sid < kSlots && !(s = slot_of(sid)); sid++) {
    }
    if (!s || !s->subs || !s->d_enc_sec || !packed_bits || packed_bits->size() != digitG) {
        *rc = -1;
        return nullptr;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaSetDevice(sid);
    std::shared_ptr<std::vector<RLWE::RGSW_ciphertext>> result;
    {
        const size_t rw = 2 * (size_t)N, gw = (size_t)digitG * 4 * N;
        std::vector<uint64_t> in(rw * digitG), out(gw * N);
        for (uint64_t j = 0; j < digitG; j++) flat_rlwe((*packed_bits)[j], &in[j * rw]);
        DevBuf din(in.size()), dout(out.size());
        cudaError_t e = din.e != cudaSuccess ? din.e : dout.e;
        if (e == cudaSuccess) e = cudaMemcpy(din.p, in.data(), in.size() * sizeof(uint64_t), cudaMemcpyHostToDevice);
        int r = e == cudaSuccess ? fheacc_homo_expand(s->ctx, din.p, s->d_enc_sec, dout.p, nullptr) : FHEACC_EIO;
        if (r == FHEACC_OK) r = fheacc_sync(s->ctx, 0);
        if (r == FHEACC_OK && cudaMemcpy(out.data(), dout.p, out.size() * sizeof(uint64_t),
                                         cudaMemcpyDeviceToHost) != cudaSuccess)
            r = FHEACC_EIO;
        if (e == cudaErrorMemoryAllocation) r = FHEACC_ENOMEM;
        cudaGetLastError();
        *rc = fpga_rc(r);
        if (r == FHEACC_OK) {
            result = std::make_shared<std::vector<RLWE::RGSW_ciphertext>>(N);
            for (int i = 0; i < N; i++) (*result)[i] = rgsw_of(&out[i * gw]);
        }
    }
    cudaSetDevice(dev);
    return result;
}

namespace {

// The lowest configured slot and its index (nullptr if none), with that
// device made current for the duration of a call.
struct SlotCall {
    Slot *s = nullptr;
    int prev = 0;
    SlotCall()
    {
        int sid = 0;
        while (sid < kSlots && !slot_of(sid)) sid++;
        if (sid == kSlots) return;
        s = slot_of(sid);
        cudaGetDevice(&prev);
        cudaSetDevice(sid);
    }
    ~SlotCall()
    {
        if (s) cudaSetDevice(prev);
        cudaGetLastError();
    }
};

}  // namespace

RLWE::RLWE_ciphertext CMUX(const RLWE::RLWE_ciphertext &c0, const RLWE::RLWE_ciphertext &c1,
                           const RLWE::RGSW_ciphertext &SEL)
{
    SlotCall sc;
    if (!sc.s || !c0.NTT_form || !c1.NTT_form) return RLWE::RLWE_ciphertext();
    const size_t rw = 2 * (size_t)N, gw = (size_t)digitG * 4 * N;
    std::vector<uint64_t> in(2 * rw), sel(gw), out(rw);
    flat_rlwe(c0, in.data());
    flat_rlwe(c1, in.data() + rw);
    flat_rgsw(SEL, sel.data());
    DevBuf din(2 * rw), dsel(gw), dout(rw);
    cudaError_t e = din.e != cudaSuccess ? din.e : dsel.e != cudaSuccess ? dsel.e : dout.e;
    if (e == cudaSuccess) e = cudaMemcpy(din.p, in.data(), in.size() * sizeof(uint64_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dsel.p, sel.data(), gw * sizeof(uint64_t), cudaMemcpyHostToDevice);
    int r = e == cudaSuccess ? fheacc_cmux_async(sc.s->ctx, din.p, din.p + rw, rw, dsel.p, 1, dout.p, 1, nullptr) : FHEACC_EIO;
    if (r == FHEACC_OK) r = fheacc_sync(sc.s->ctx, 0);
    if (r == FHEACC_OK && cudaMemcpy(out.data(), dout.p, rw * sizeof(uint64_t), cudaMemcpyDeviceToHost) != cudaSuccess)
        r = FHEACC_EIO;
    return r == FHEACC_OK ? rlwe_of(out.data()) : RLWE::RLWE_ciphertext();
}

RLWE::RLWE_ciphertext blind_rotate(const RLWE::RLWE_ciphertext &c_in, const bool forward,
                                   const std::vector<RLWE::RGSW_ciphertext> &C)
{
    SlotCall sc;
    if (!sc.s || C.size() != (size_t)digitN) return RLWE::RLWE_ciphertext();
    const size_t rw = 2 * (size_t)N, gw = (size_t)digitG * 4 * N;
    std::vector<uint64_t> in(rw), rg(gw * C.size()), out(rw);
    flat_rlwe(c_in, in.data());
    for (size_t i = 0; i < C.size(); i++) flat_rgsw(C[i], &rg[i * gw]);
    DevBuf din(rw), drg(rg.size()), dout(rw);
    cudaError_t e = din.e != cudaSuccess ? din.e : drg.e != cudaSuccess ? drg.e : dout.e;
    if (e == cudaSuccess) e = cudaMemcpy(din.p, in.data(), rw * sizeof(uint64_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(drg.p, rg.data(), rg.size() * sizeof(uint64_t), cudaMemcpyHostToDevice);
    int r = e == cudaSuccess ? FHEACC_OK : FHEACC_EIO;
    // the CPU path moves the input to the NTT domain first (RLWE.cpp:830)
    if (r == FHEACC_OK && !c_in.NTT_form) r = fheacc_ntt_forward(sc.s->ctx, din.p, 2, nullptr);
    if (r == FHEACC_OK) r = fheacc_rlwe_blind_rotate_async(sc.s->ctx, din.p, drg.p, forward ? 1 : 0, dout.p, 1, nullptr);
    if (r == FHEACC_OK) r = fheacc_sync(sc.s->ctx, 0);
    if (r == FHEACC_OK && cudaMemcpy(out.data(), dout.p, rw * sizeof(uint64_t), cudaMemcpyDeviceToHost) != cudaSuccess)
        r = FHEACC_EIO;
    return r == FHEACC_OK ? rlwe_of(out.data()) : RLWE::RLWE_ciphertext();
}

void set_issue_flags(uint32_t flags) { g_flags = flags & (FHEACC_FLAG_FPGA_COMPAT | FHEACC_FLAG_FPGA_X1); }

fheacc_ctx *context(const int slot_id)
{
    Slot *s = slot_of(slot_id);
    return s ? s->ctx : nullptr;
}

int release(const int slot_id)
{
    if (slot_id < 0 || slot_id >= kSlots) return -1;
    Slot &s = g_slot[slot_id];
    if (s.d_enc_sec) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaSetDevice(slot_id);
        cudaFree(s.d_enc_sec);
        cudaSetDevice(dev);
    }
    if (s.ctx) fheacc_destroy(s.ctx);
    s = Slot();
    return 0;
}

}  // namespace GPU
