// graph.cu -- batched bootstraps of several parameter sets in one CUDA-graph
// launch, and the launch-shape autotuner.
//
// The reference has no counterpart: its FPGA runtime serves one parameter set
// per process (params.h globals) and issues gates one instruction at a time
// (myfpga.cpp:1446-1492). Here a graph holds any number of batched gate
// bootstraps over any number of contexts (parameter sets) of one device. At
// the first launch the batches are captured in the order they were added, on
// one branch; with FHEACC_GRAPH_CONCURRENT each context gets its own branch (a
// stream forked from the capture stream) and the branches join at the end.
// Both blind-rotation kernels are persistent grids sized to fill the GPU, so
// concurrent branches share SMs unevenly and finish later than the serial
// order for throughput-bound batches; they help when the batches are small.
// The graph owns the scratch of every context, so later calls on the same
// contexts cannot move memory the graph refers to. Replays are one
// cudaGraphLaunch.
//
// The autotuner times the blind rotation's launch options (register budget,
// CTAs per SM, ciphertexts per CTA) on a synthetic batch of the caller's size
// with the context's keys and keeps the fastest.
#include "ctx.hpp"
#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <vector>

using namespace fheacc;

struct fheacc_graph {
    struct Item {
        Context *c;
        const uint64_t *c1, *c2;
        const int32_t *gates;
        size_t count;
        uint64_t *out;
    };
    std::vector<Item> items;
    std::vector<void *> scratch;   // per branch: accumulators, extracted RLWEs
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int device = -1;
    uint32_t flags = 0;
    std::string err;

    int fail(int rc, const std::string &m)
    {
        err = m;
        return rc;
    }
    void drop()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
        for (void *p : scratch) cudaFree(p);
        scratch.clear();
    }
    int capture();
};

int fheacc_graph::capture()
{
    drop();
    // branches: one per context, in order of first appearance
    std::vector<Context *> order;
    std::map<Context *, size_t> most;
    for (const Item &it : items) {
        if (!most.count(it.c)) order.push_back(it.c);
        most[it.c] = std::max(most[it.c], it.count);
    }
    for (Context *c : order) {
        void *a = nullptr, *x = nullptr;
        const size_t m = std::max<size_t>(most[c], 1);
        if (cudaMalloc(&a, bootstrap_accs_bytes(*c, m)) != cudaSuccess ||
            cudaMalloc(&x, bootstrap_extract_bytes(*c, m)) != cudaSuccess) {
            cudaGetLastError();
            if (a) cudaFree(a);
            drop();
            return fail(FHEACC_ENOMEM, "graph scratch allocation failed");
        }
        scratch.push_back(a);
        scratch.push_back(x);
    }
    cudaStream_t cap = nullptr;
    std::vector<cudaStream_t> br(order.size(), nullptr);
    std::vector<cudaEvent_t> join(order.size(), nullptr);
    cudaEvent_t fork = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
    for (size_t b = 0; b < order.size() && e == cudaSuccess; b++) {
        e = cudaStreamCreateWithFlags(&br[b], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&join[b], cudaEventDisableTiming);
    }
    int rc = FHEACC_OK;
    bool capturing = false;
    if (e == cudaSuccess) e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeRelaxed);
    if (e == cudaSuccess) {
        capturing = true;
        e = cudaEventRecord(fork, cap);
    }
    const bool concurrent = (flags & FHEACC_GRAPH_CONCURRENT) != 0;
    auto ctx_index = [&](const Context *c) { return (size_t)(std::find(order.begin(), order.end(), c) - order.begin()); };
    if (!concurrent) {
        // one branch: every batch in the order added, on the capture stream
        for (const Item &it : items) {
            if (e != cudaSuccess || rc) break;
            const size_t b = ctx_index(it.c);
            rc = bootstrap_device_with(*it.c, it.c1, it.c2, it.gates, it.count, it.out, 0, scratch[2 * b],
                                       scratch[2 * b + 1], cap);
            if (rc) err = std::string("capture: ") + fheacc_last_error(reinterpret_cast<fheacc_ctx *>(it.c));
        }
    }
    for (size_t b = 0; concurrent && b < order.size() && e == cudaSuccess && !rc; b++) {
        e = cudaStreamWaitEvent(br[b], fork, 0);
        for (const Item &it : items) {
            if (it.c != order[b] || e != cudaSuccess || rc) continue;
            rc = bootstrap_device_with(*it.c, it.c1, it.c2, it.gates, it.count, it.out, 0, scratch[2 * b],
                                       scratch[2 * b + 1], br[b]);
            if (rc) err = std::string("capture: ") + fheacc_last_error(reinterpret_cast<fheacc_ctx *>(it.c));
        }
        if (e == cudaSuccess && !rc) e = cudaEventRecord(join[b], br[b]);
        if (e == cudaSuccess && !rc) e = cudaStreamWaitEvent(cap, join[b], 0);
    }
    if (capturing) {
        cudaGraph_t g = nullptr;
        const cudaError_t e2 = cudaStreamEndCapture(cap, &g);
        if (e == cudaSuccess) e = e2;
        if (e == cudaSuccess && !rc) graph = g;
        else if (g) cudaGraphDestroy(g);
    }
    if (e == cudaSuccess && !rc) e = cudaGraphInstantiate(&exec, graph, 0);
    for (size_t b = 0; b < order.size(); b++) {
        if (join[b]) cudaEventDestroy(join[b]);
        if (br[b]) cudaStreamDestroy(br[b]);
    }
    if (fork) cudaEventDestroy(fork);
    if (cap) cudaStreamDestroy(cap);
    if (e != cudaSuccess && !rc) rc = fail(FHEACC_EIO, std::string("graph capture: ") + cudaGetErrorString(e));
    if (rc) {
        cudaGetLastError();
        drop();
    }
    return rc;
}

namespace {

// SplitMix64: the synthetic batches of the autotuner.
uint64_t mix64(uint64_t &s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

}  // namespace

extern "C" {

int fheacc_graph_create(fheacc_graph **out, uint32_t flags)
{
    if (!out) return FHEACC_EINVAL;
    *out = nullptr;
    if (flags & ~(uint32_t)FHEACC_GRAPH_CONCURRENT) return FHEACC_EINVAL;
    fheacc_graph *g = new (std::nothrow) fheacc_graph();
    if (!g) return FHEACC_ENOMEM;
    g->flags = flags;
    *out = g;
    return FHEACC_OK;
}

int fheacc_graph_add_bootstrap(fheacc_graph *g, fheacc_ctx *ctx, const uint64_t *d_c1, const uint64_t *d_c2,
                               const int32_t *d_gates, size_t count, uint64_t *d_out)
{
    if (!g) return FHEACC_EINVAL;
    if (!ctx) return g->fail(FHEACC_EINVAL, "null context");
    if (count && (!d_c1 || !d_c2 || !d_gates || !d_out)) return g->fail(FHEACC_EINVAL, "null buffer");
    Context &c = *reinterpret_cast<Context *>(ctx);
    if (g->device >= 0 && g->device != c.device) return g->fail(FHEACC_EINVAL, "contexts of one graph share a device");
    if (c.wide ? !c.d_btkey64 || !c.d_kskey64 : !c.d_btkey || !c.d_kskey)
        return g->fail(FHEACC_ENOKEY, "keys must be uploaded before the context joins a graph");
    g->device = c.device;
    if (!count) return FHEACC_OK;
    DeviceGuard dg(c.device);
    g->drop();   // re-captured at the next launch
    g->items.push_back({&c, d_c1, d_c2, d_gates, count, d_out});
    return FHEACC_OK;
}

int fheacc_graph_launch(fheacc_graph *g, void *stream)
{
    if (!g) return FHEACC_EINVAL;
    if (g->items.empty()) return FHEACC_OK;
    DeviceGuard dg(g->device);
    if (!g->exec) {
        const int rc = g->capture();
        if (rc) return rc;
    }
    const cudaError_t e = cudaGraphLaunch(g->exec, (cudaStream_t)stream);
    return e == cudaSuccess ? FHEACC_OK : g->fail(FHEACC_EIO, std::string("graph launch: ") + cudaGetErrorString(e));
}

size_t fheacc_graph_batches(const fheacc_graph *g) { return g ? g->items.size() : 0; }

const char *fheacc_graph_last_error(const fheacc_graph *g) { return g ? g->err.c_str() : "null graph"; }

int fheacc_graph_destroy(fheacc_graph *g)
{
    if (!g) return FHEACC_OK;
    if (g->device >= 0) {
        DeviceGuard dg(g->device);
        g->drop();
    }
    delete g;
    return FHEACC_OK;
}

int fheacc_autotune(fheacc_ctx *ctx, size_t count, fheacc_tune_trial *trials, int max_trials, int *n_trials)
{
    if (!ctx) return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    if (count == 0 || count > ((size_t)1 << 22)) return c.fail(FHEACC_EINVAL, "autotune: count must be 1..4M");
    if (c.wide ? !c.d_btkey64 || !c.d_kskey64 : !c.d_btkey || !c.d_kskey)
        return c.fail(FHEACC_ENOKEY, "autotune: keys must be uploaded");
    DeviceGuard dg(c.device);
    // synthetic batch: uniform LWE ciphertexts mod q, the six gates in turn
    const size_t w = (size_t)c.p.n + 1;
    std::vector<uint64_t> h(2 * count * w);
    uint64_t seed = 0x5EEDF00DULL + count;
    for (uint64_t &x : h) x = mix64(seed) % c.p.q;
    std::vector<int32_t> hg(count);
    for (size_t i = 0; i < count; i++) hg[i] = (int32_t)(i % 6);
    const size_t in_bytes = h.size() * sizeof(uint64_t), out_bytes = count * w * sizeof(uint64_t);
    char *d = nullptr;
    const size_t accs = bootstrap_accs_bytes(c, count), ext = bootstrap_extract_bytes(c, count);
    const size_t off_g = in_bytes, off_o = (off_g + count * 4 + 255) / 256 * 256, off_a = (off_o + out_bytes + 255) / 256 * 256,
                 off_x = (off_a + accs + 255) / 256 * 256;
    if (cudaMalloc(&d, off_x + ext) != cudaSuccess) {
        cudaGetLastError();
        return c.fail(FHEACC_ENOMEM, "autotune scratch");
    }
    cudaError_t e = cudaMemcpy(d, h.data(), in_bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d + off_g, hg.data(), count * 4, cudaMemcpyHostToDevice);
    const uint64_t *d1 = (const uint64_t *)d, *d2 = d1 + count * w;
    const int32_t *dgates = (const int32_t *)(d + off_g);
    uint64_t *dout = (uint64_t *)(d + off_o);
    // candidates: (register budget for 3 CTAs/SM, CTAs per SM cap, group cap,
    // steps per bucket of the step window, pipelines per CTA)
    struct Cand {
        int regs3, ctas, group, window, pipes;
    };
    std::vector<Cand> cands;
    if (c.wide) {
        for (int pipes : {2, 3, 1})
            for (int window : {-1, 0}) cands.push_back({-1, 0, 0, window, pipes});
        cands.push_back({-1, 0, 4, -1, 2});
        cands.push_back({-1, 1, 0, -1, 1});
    } else {
        for (int group : {0, 6, 12}) cands.push_back({-1, 0, group, -1, 3});
        cands.push_back({-1, 0, 0, -1, 2});
        for (int regs3 : {0, 1})
            for (int group : {0, 12}) cands.push_back({regs3, 0, group, -1, 1});
    }
    const Tuning saved = c.tune;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    int rc = e == cudaSuccess ? FHEACC_OK : c.cuda_fail(e, "autotune setup");
    float best = 1e30f;
    Tuning best_t = saved;
    int nt = 0;
    for (const Cand &k : cands) {
        if (rc) break;
        c.tune.br_regs_for_3 = k.regs3;
        c.tune.br_ctas_per_sm = k.ctas;
        c.tune.br_group = k.group;
        c.tune.br_window = k.window;
        c.tune.br_pipes = k.pipes;
        float t = 1e30f;
        for (int rep = 0; rep < 3 && !rc; rep++) {
            cudaEventRecord(e0, c.stream);
            rc = bootstrap_device_with(c, d1, d2, dgates, count, dout, 0, d + off_a, d + off_x, c.stream);
            cudaEventRecord(e1, c.stream);
            if (!rc) {
                e = cudaEventSynchronize(e1);
                if (e != cudaSuccess) rc = c.cuda_fail(e, "autotune trial");
            }
            float ms = 0;
            if (!rc && rep > 0 && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess) t = std::min(t, ms);
        }
        if (rc) break;
        if (trials && nt < max_trials) trials[nt] = {k.regs3, k.ctas, k.group, k.window, k.pipes, t};
        nt++;
        if (t < best) {
            best = t;
            best_t = c.tune;
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(d);
    c.tune = rc ? saved : best_t;
    if (n_trials) *n_trials = nt;
    return rc;
}

}  // extern "C"
