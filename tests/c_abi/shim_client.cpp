// Drives the GPU:: backend (3rd_gen_fhe_acc_gb300/integration/gpu_backend.cpp)
// the way the runtime's FPGA tests drive FPGA:: (test.cpp:2013-3538):
// configure slot 0 from the runtime's globals, upload and read back the keys,
// bootstrap through the fixed-width calls, expand, CMUX and blind-rotate. Keys and ciphertexts come from
// libfheacc's seeded host generator; every bootstrap output is decrypted and
// compared word for word with libfheacc's own host-buffer call, and the expand
// outputs with the C ABI's device calls. Built against the runtime's headers
// or the stand-ins in tests/c_abi/runtime_api. Prints "shim ok" and exits 0;
// a failed check prints its name and exits 1.
#include "gpu_backend.h"

#include <cstdio>
#include <cstdlib>
#include <cuda_runtime.h>

int n;
ciphertext_t q;
int N;
uint16_t digitN;
ciphertext_t E_rlwe, Q, iN, ROU, BGbits, digitG, Br, digitR, Bks, digitKS, Bks_R_bits, digitKS_R;
ciphertext_t gate_constant[6];

#define CHECK(cond)                                                  \
    do {                                                             \
        if (!(cond)) {                                               \
            std::printf("FAILED line %d: %s\n", __LINE__, #cond);    \
            std::exit(1);                                            \
        }                                                            \
    } while (0)

static fheacc_params P;

static int truth(int g, int a, int b)
{
    switch (g) {
    case OR: return a | b;
    case AND: return a & b;
    case NOR: return !(a | b);
    case NAND: return !(a & b);
    case XOR: return a ^ b;
    default: return !(a ^ b);
    }
}

static RLWE::RLWE_ciphertext rlwe_of(const uint64_t *w)
{
    RLWE::RLWE_ciphertext c;
    for (int i = 0; i < N; i++) {
        c.a[i] = w[i];
        c.b[i] = w[N + i];
    }
    return c;
}

static RLWE::RGSW_ciphertext rgsw_of(const uint64_t *w)
{
    RLWE::RGSW_ciphertext g;
    g.c_text.resize(digitG);
    for (uint64_t h = 0; h < digitG; h++)
        for (int r = 0; r < 2; r++) g.c_text[h].push_back(rlwe_of(w + (h * 2 + r) * 2 * (size_t)N));
    return g;
}

static LWE::LWE_ciphertext lwe_of(const uint64_t *w)
{
    LWE::LWE_ciphertext c;
    for (int i = 0; i < n; i++) c.a[i] = w[i];
    c.b = w[n];
    return c;
}

static std::vector<uint64_t> flat(const LWE::LWE_ciphertext &c)
{
    std::vector<uint64_t> w(c.a.begin(), c.a.begin() + n);
    w.push_back(c.b);
    return w;
}

// fheacc_bootstrap on the same inputs, through the backend's context
static void check_same(const std::vector<LWE::LWE_ciphertext> &c1, const std::vector<LWE::LWE_ciphertext> &c2,
                       const std::vector<GATES> &g, const std::vector<LWE::LWE_ciphertext> &got, uint32_t flags)
{
    const size_t k = got.size(), w = (size_t)n + 1;
    std::vector<uint64_t> a, b, o(k * w);
    std::vector<int32_t> gg;
    for (size_t i = 0; i < k; i++) {
        auto x = flat(c1[i]), y = flat(c2[i]);
        a.insert(a.end(), x.begin(), x.end());
        b.insert(b.end(), y.begin(), y.end());
        gg.push_back((int32_t)g[i]);
    }
    CHECK(fheacc_bootstrap(GPU::context(0), a.data(), b.data(), gg.data(), k, o.data(), flags) == FHEACC_OK);
    for (size_t i = 0; i < k; i++) CHECK(flat(got[i]) == std::vector<uint64_t>(o.begin() + i * w, o.begin() + (i + 1) * w));
}

static void check_decrypts(const std::vector<uint64_t> &lsk, const std::vector<LWE::LWE_ciphertext> &out,
                           const std::vector<GATES> &g, const std::vector<uint8_t> &x, const std::vector<uint8_t> &y)
{
    for (size_t i = 0; i < out.size(); i++) {
        uint8_t m = 9;
        auto w = flat(out[i]);
        CHECK(fheacc_lwe_decrypt(&P, lsk.data(), w.data(), 1, &m) == FHEACC_OK);
        CHECK(m == truth(g[i], x[i], y[i]));
    }
}

int main()
{
    CHECK(fheacc_params_preset(0, &P) == FHEACC_OK);
    P.n = 32;   // a reduced LWE dimension keeps key generation quick; the ring is unchanged
    CHECK(fheacc_params_derive(&P) == FHEACC_OK);
    n = P.n; q = P.q; N = P.N; Q = P.Q; iN = P.iN; ROU = P.ROU; E_rlwe = P.E_rlwe;
    BGbits = P.BG_bits; digitG = P.digitG; Br = P.Br; digitR = P.digitR; Bks = P.Bks; digitKS = P.digitKS;
    Bks_R_bits = P.Bks_R_bits; digitKS_R = P.digitKS_R;
    digitN = 0;
    while ((1 << digitN) < N) digitN++;
    for (int g = 0; g < 6; g++) gate_constant[g] = P.gate_constant[g];

    std::vector<uint64_t> lsk(n), rsk(N), bt(fheacc_bootstrap_key_words(&P)), ks(fheacc_lwe_ks_key_words(&P)),
        subs(fheacc_subs_key_words(&P));
    CHECK(fheacc_keygen_lwe_sk(&P, 11, lsk.data()) == FHEACC_OK);
    CHECK(fheacc_keygen_rlwe_sk(&P, 12, rsk.data()) == FHEACC_OK);
    CHECK(fheacc_keygen_bootstrap_key(&P, 13, lsk.data(), rsk.data(), bt.data(), 0) == FHEACC_OK);
    CHECK(fheacc_keygen_lwe_ks_key(&P, 14, rsk.data(), lsk.data(), ks.data(), 0) == FHEACC_OK);
    CHECK(fheacc_keygen_subs_key(&P, 15, rsk.data(), subs.data(), 0) == FHEACC_OK);

    // the runtime's key objects
    const size_t gw = (size_t)digitG * 4 * N;
    RLWE::bootstrap_key bk;
    bk.btkey.resize(Br);
    for (uint64_t r = 0; r < Br; r++) {
        bk.btkey[r].resize(digitR);
        for (uint64_t j = 0; j < digitR; j++)
            for (int i = 0; i < n; i++) bk.btkey[r][j].push_back(rgsw_of(&bt[((r * digitR + j) * n + i) * gw]));
    }
    LWE::keyswitch_key kk;
    kk.kskey.resize(Bks);
    for (uint64_t d = 0; d < Bks; d++) {
        kk.kskey[d].resize(digitKS);
        for (uint64_t j = 0; j < digitKS; j++)
            for (int i = 0; i < N; i++) kk.kskey[d][j].push_back(lwe_of(&ks[((d * digitKS + j) * N + i) * (n + 1)]));
    }
    application::substitute_key sk;
    sk.subs_key.resize(digitN);
    for (int l = 0; l < digitN; l++)
        for (uint64_t i = 0; i < digitKS_R; i++)
            sk.subs_key[l].RLWE_kskey.push_back(rlwe_of(&subs[(l * digitKS_R + i) * 2 * (size_t)N]));

    CHECK(GPU::OCL_config_wr_rd(0) == 0);
    CHECK(GPU::BAR1_ROU_table_1k_wr(0) == 0);
    CHECK(GPU::dma_write_bootstrap_key(0, bk) == 0);
    CHECK(GPU::dma_write_subs_key(0, sk) == 0);

    // slot check, byte compare and the read-back verifiers: the keys just
    // uploaded compare equal, a copy with one word changed does not
    CHECK(GPU::check_slot_config(0) == 0 && GPU::check_slot_config(-1) == 1 && GPU::check_slot_config(4096) == 1);
    {
        uint8_t u[8] = {1, 2, 3, 4, 5, 6, 7, 8}, v[8] = {1, 0, 3, 4, 0, 6, 7, 0};
        CHECK(GPU::buffer_compare(u, v, 8) == 3 && GPU::buffer_compare(u, u, 8) == 0);
    }
    CHECK(GPU::dma_read_compare_bootstrap_key(0, bk) == 0);
    CHECK(GPU::dma_read_compare_subs_key(0, sk) == 0);
    {
        RLWE::bootstrap_key bad = bk;
        bad.btkey[3][1][7].c_text[2][1].a[5] ^= 1;
        CHECK(GPU::dma_read_compare_bootstrap_key(0, bad) == -1);
        application::substitute_key bad_sk = sk;
        bad_sk.subs_key[4].RLWE_kskey[1].b[9] ^= 1;
        CHECK(GPU::dma_read_compare_subs_key(0, bad_sk) == -1);
        CHECK(GPU::dma_read_compare_bootstrap_key(1000, bk) == -1);
    }

    // twelve gates of random bits
    const int K = 12;
    std::vector<uint8_t> bits(2 * K), x(K), y(K);
    for (int i = 0; i < 2 * K; i++) bits[i] = (uint8_t)((i * 7 + 3) % 5 % 2);
    std::vector<uint64_t> cw(2 * K * (size_t)(n + 1));
    CHECK(fheacc_lwe_encrypt(&P, 16, lsk.data(), bits.data(), 2 * K, cw.data()) == FHEACC_OK);
    std::vector<LWE::LWE_ciphertext> c1, c2;
    std::vector<GATES> g;
    for (int i = 0; i < K; i++) {
        c1.push_back(lwe_of(&cw[i * (size_t)(n + 1)]));
        c2.push_back(lwe_of(&cw[(K + i) * (size_t)(n + 1)]));
        x[i] = bits[i];
        y[i] = bits[K + i];
        g.push_back((GATES)(i % 6));
    }
    int rc = 1;
    const pci_bar_handle_t bar = 0;
    // x4 (the 4-gate call the FPGA tests use), then the other widths
    auto sub = [&](const std::vector<LWE::LWE_ciphertext> &v, int k) {
        return std::vector<LWE::LWE_ciphertext>(v.begin(), v.begin() + k);
    };
    std::vector<GATES> g4(g.begin(), g.begin() + 4);
    auto o4 = GPU::fpga_eval_bootstrap_x4(sub(c1, 4), sub(c2, 4), kk, g4, bar, &rc, -1);
    CHECK(rc == 0);
    check_decrypts(lsk, o4, g4, x, y);
    check_same(sub(c1, 4), sub(c2, 4), g4, o4, 0);
    auto o8 = GPU::fpga_eval_bootstrap_x8(sub(c1, 8), sub(c2, 8), kk, g, bar, &rc, -1);
    CHECK(rc == 0 && o8.size() == 8);
    check_decrypts(lsk, o8, g, x, y);
    auto o12 = GPU::fpga_eval_bootstrap_x12(c1, c2, kk, g, bar, &rc, -1);
    CHECK(rc == 0 && o12.size() == 12);
    check_decrypts(lsk, o12, g, x, y);
    auto o10 = GPU::fpga_eval_bootstrap_x16(sub(c1, 10), sub(c2, 10), kk, g, bar, &rc, -1);
    CHECK(rc == 0 && o10.size() == 10);
    check_same(sub(c1, 10), sub(c2, 10), std::vector<GATES>(g.begin(), g.begin() + 10), o10, 0);
    // sizes the FPGA calls refuse, and c1 == c2
    GPU::fpga_eval_bootstrap_x16(c1, c2, kk, g, bar, &rc, -1);
    CHECK(rc == -1);
    GPU::fpga_eval_bootstrap_x4(sub(c1, 3), sub(c2, 3), kk, g, bar, &rc, -1);
    CHECK(rc == -1);
    GPU::fpga_eval_bootstrap_x4(sub(c1, 4), sub(c1, 4), kk, g4, bar, &rc, -1);
    CHECK(rc == -1);
    // x1 in the CPU order and in x1's own FPGA order
    LWE::LWE_ciphertext o1 = GPU::fpga_eval_bootstrap_x1(c1[5], c2[5], kk, g[5], bar, &rc, -1);
    CHECK(rc == 0);
    check_decrypts(lsk, {o1}, {g[5]}, {x[5]}, {y[5]});
    check_same({c1[5]}, {c2[5]}, {g[5]}, {o1}, 0);
    // the RLWE::eval_bootstrap-compatible call: the same words as the CPU-order x1
    LWE::LWE_ciphertext oe = GPU::eval_bootstrap(c1[5], c2[5], bk, kk, g[5]);
    check_same({c1[5]}, {c2[5]}, {g[5]}, {oe}, 0);
    {
        // c1 == c2: a default-constructed (all-zero) ciphertext, as the FPGA calls return on error
        const LWE::LWE_ciphertext z = GPU::eval_bootstrap(c1[5], c1[5], bk, kk, g[5]);
        bool zero = z.b == 0;
        for (int i = 0; i < n; i++) zero = zero && z.a[i] == 0;
        CHECK(zero);
    }
    GPU::set_issue_flags(FHEACC_FLAG_FPGA_X1);
    LWE::LWE_ciphertext o1x = GPU::fpga_eval_bootstrap_x1(c1[5], c2[5], kk, g[5], bar, &rc, -1);
    CHECK(rc == 0);
    check_same({c1[5]}, {c2[5]}, {g[5]}, {o1x}, FHEACC_FLAG_FPGA_X1);
    GPU::set_issue_flags(0);

    // expand_RLWE and homo_expand against the C ABI's device calls
    std::vector<uint64_t> msg(N), packed(digitG * 2 * (size_t)N), rgsw(gw);
    for (int i = 0; i < N; i++) msg[i] = (uint64_t)(i * 977 + 5) % Q;
    for (uint64_t j = 0; j < digitG; j++)
        CHECK(fheacc_rlwe_encrypt(&P, 100 + j, rsk.data(), msg.data(), &packed[j * 2 * (size_t)N]) == FHEACC_OK);
    CHECK(fheacc_rgsw_encrypt(&P, 41, rsk.data(), msg.data(), rgsw.data()) == FHEACC_OK);
    CHECK(GPU::dma_read_compare_RGSW_enc_sk(0, rgsw_of(rgsw.data())) == -1);   // not uploaded yet
    CHECK(GPU::dma_write_RGSW_enc_sk(0, rgsw_of(rgsw.data())) == 0);
    CHECK(GPU::dma_read_compare_RGSW_enc_sk(0, rgsw_of(rgsw.data())) == 0);
    {
        std::vector<uint64_t> bad(rgsw);
        bad[gw / 2 + 3] ^= 1;
        CHECK(GPU::dma_read_compare_RGSW_enc_sk(0, rgsw_of(bad.data())) == -1);
    }
    auto ex = GPU::fpga_expand_RLWE(rlwe_of(packed.data()), bar, &rc, -1, -1);
    CHECK(rc == 0 && ex && ex->size() == (size_t)N);
    // the reference's DMA-issue variants of expand_RLWE give the same RLWEs
    auto ex_cont = GPU::fpga_expand_RLWE_cont_rd_wr(rlwe_of(packed.data()), bar, &rc, -1, -1);
    CHECK(rc == 0 && ex_cont && ex_cont->size() == (size_t)N);
    auto ex_batch = GPU::fpga_expand_RLWE_batch_rd_wr(rlwe_of(packed.data()), bar, &rc, -1, -1);
    CHECK(rc == 0 && ex_batch && ex_batch->size() == (size_t)N);
    for (int i = 0; i < N; i++)
        for (int k = 0; k < N; k++) {
            CHECK((*ex_cont)[i].a[k] == (*ex)[i].a[k] && (*ex_cont)[i].b[k] == (*ex)[i].b[k]);
            CHECK((*ex_batch)[i].a[k] == (*ex)[i].a[k] && (*ex_batch)[i].b[k] == (*ex)[i].b[k]);
        }
    auto packs = std::make_unique<std::vector<RLWE::RLWE_ciphertext>>();
    for (uint64_t j = 0; j < digitG; j++) packs->push_back(rlwe_of(&packed[j * 2 * (size_t)N]));
    auto he = GPU::fpga_homo_expand(packs, bar, &rc, -1, -1);
    CHECK(rc == 0 && he && he->size() == (size_t)N);
    {
        const size_t rw = 2 * (size_t)N;
        uint64_t *d_in = nullptr, *d_out = nullptr, *d_sec = nullptr;
        CHECK(cudaMalloc(&d_in, packed.size() * 8) == cudaSuccess);
        CHECK(cudaMalloc(&d_out, gw * N * 8) == cudaSuccess);
        CHECK(cudaMalloc(&d_sec, gw * 8) == cudaSuccess);
        CHECK(cudaMemcpy(d_in, packed.data(), packed.size() * 8, cudaMemcpyHostToDevice) == cudaSuccess);
        CHECK(cudaMemcpy(d_sec, rgsw.data(), gw * 8, cudaMemcpyHostToDevice) == cudaSuccess);
        std::vector<uint64_t> want(gw * N);
        CHECK(fheacc_expand_rlwe(GPU::context(0), d_in, d_out, nullptr) == FHEACC_OK);
        CHECK(fheacc_sync(GPU::context(0), 0) == FHEACC_OK);
        CHECK(cudaMemcpy(want.data(), d_out, rw * N * 8, cudaMemcpyDeviceToHost) == cudaSuccess);
        for (int i = 0; i < N; i++)
            for (int k = 0; k < N; k++)
                CHECK((*ex)[i].a[k] == want[i * rw + k] && (*ex)[i].b[k] == want[i * rw + N + k]);
        CHECK(fheacc_homo_expand(GPU::context(0), d_in, d_sec, d_out, nullptr) == FHEACC_OK);
        CHECK(fheacc_sync(GPU::context(0), 0) == FHEACC_OK);
        CHECK(cudaMemcpy(want.data(), d_out, gw * N * 8, cudaMemcpyDeviceToHost) == cudaSuccess);
        for (int i = 0; i < N; i++)
            for (uint64_t h = 0; h < digitG; h++)
                for (int r = 0; r < 2; r++) {
                    const uint64_t *w = &want[i * gw + (h * 2 + r) * rw];
                    const RLWE::RLWE_ciphertext &c = (*he)[i].c_text[h][r];
                    for (int k = 0; k < N; k++) CHECK(c.a[k] == w[k] && c.b[k] == w[N + k]);
                }
        // CMUX and blind_rotate with the RLWE:: signatures, against the C ABI's
        // device calls on the same words; a time-domain input of blind_rotate
        // gives what its NTT-domain form gives
        const RLWE::RLWE_ciphertext c0 = rlwe_of(&packed[0]), c1 = rlwe_of(&packed[rw]);
        const RLWE::RGSW_ciphertext sel = rgsw_of(rgsw.data());
        const RLWE::RLWE_ciphertext mux = GPU::CMUX(c0, c1, sel);
        CHECK(fheacc_cmux_async(GPU::context(0), d_in, d_in + rw, rw, d_sec, 1, d_out, 1, nullptr) == FHEACC_OK);
        CHECK(fheacc_sync(GPU::context(0), 0) == FHEACC_OK);
        CHECK(cudaMemcpy(want.data(), d_out, rw * 8, cudaMemcpyDeviceToHost) == cudaSuccess);
        for (int k = 0; k < N; k++) CHECK(mux.a[k] == want[k] && mux.b[k] == want[N + k]);
        std::vector<RLWE::RGSW_ciphertext> ctl(digitN, sel);
        uint64_t *d_ctl = nullptr;
        CHECK(cudaMalloc(&d_ctl, gw * digitN * 8) == cudaSuccess);
        for (int i = 0; i < digitN; i++)
            CHECK(cudaMemcpy(d_ctl + i * gw, rgsw.data(), gw * 8, cudaMemcpyHostToDevice) == cudaSuccess);
        const RLWE::RLWE_ciphertext rot = GPU::blind_rotate(c0, true, ctl);
        CHECK(fheacc_rlwe_blind_rotate_async(GPU::context(0), d_in, d_ctl, 1, d_out, 1, nullptr) == FHEACC_OK);
        CHECK(fheacc_sync(GPU::context(0), 0) == FHEACC_OK);
        CHECK(cudaMemcpy(want.data(), d_out, rw * 8, cudaMemcpyDeviceToHost) == cudaSuccess);
        for (int k = 0; k < N; k++) CHECK(rot.a[k] == want[k] && rot.b[k] == want[N + k]);
        CHECK(fheacc_ntt_inverse(GPU::context(0), d_in, 2, nullptr) == FHEACC_OK);   // c0 to the time domain
        CHECK(fheacc_sync(GPU::context(0), 0) == FHEACC_OK);
        std::vector<uint64_t> t0(rw);
        CHECK(cudaMemcpy(t0.data(), d_in, rw * 8, cudaMemcpyDeviceToHost) == cudaSuccess);
        RLWE::RLWE_ciphertext c0t = rlwe_of(t0.data());
        c0t.NTT_form = false;
        const RLWE::RLWE_ciphertext rot_t = GPU::blind_rotate(c0t, true, ctl);
        for (int k = 0; k < N; k++) CHECK(rot_t.a[k] == rot.a[k] && rot_t.b[k] == rot.b[k]);
        CHECK(GPU::blind_rotate(c0, true, std::vector<RLWE::RGSW_ciphertext>(digitN - 1, sel)).a[0] == 0);
        cudaFree(d_ctl);
        cudaFree(d_in);
        cudaFree(d_out);
        cudaFree(d_sec);
    }
    CHECK(GPU::release(0) == 0);
    std::printf("shim ok\n");
    return 0;
}
