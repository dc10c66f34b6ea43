// server.cu -- continuous-batching request loop over the gate-bootstrapping
// kernels (host code; the reference runtime has no serving layer, its FPGA
// driver issues one fixed-width batch at a time, myfpga.cpp:1130-1660).
//
// A request is a small gate circuit over LWE ciphertexts: num_inputs input
// ciphertexts, then num_gates gates, gate g computing node num_inputs + g =
// gate_type[g](node in1[g], node in2[g]) with eval_bootstrap semantics; its
// result is the last num_outputs nodes. A PSI equality query (32 XNOR gates
// and a 31-gate AND tree per server item) is one such circuit.
//
// Every ciphertext of an admitted request -- inputs, intermediates, outputs --
// lives in one device pool, in a contiguous range of slots reserved at
// admission. A request is admitted when the pool has room for all its nodes
// (admission by free device memory); otherwise it waits, in arrival order.
// A worker thread runs rounds: it gathers every gate, of every admitted
// request, whose inputs are ready, up to max_batch, and runs them as ONE
// batched bootstrap reading and writing the pool through index arrays. Requests
// that arrive while a round is on the GPU are admitted meanwhile and join the
// next round, so their gates share launches with the gates of older requests.
// Keys stay resident in the context; only index arrays go to the device per
// round, and only finished outputs come back.
#include "ctx.hpp"
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

namespace fheacc {

namespace {

double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Request {
    uint64_t id = 0;
    uint32_t num_inputs = 0, num_gates = 0, num_outputs = 0;
    std::vector<int32_t> type;
    std::vector<uint32_t> in1, in2;
    std::vector<uint64_t> inputs;   // host copy of the input ciphertexts
    uint64_t *out_host = nullptr;
    uint32_t base = 0;              // first pool slot
    std::vector<uint8_t> state;     // per gate: 0 waiting, 1 in flight, 2 done
    uint32_t next_scan = 0;         // gates below this are issued or done
    uint32_t done = 0;
    double t_submit = 0, t_admit = 0, t_done = 0;
    int status = FHEACC_OK;
};

}  // namespace

// One in-flight round: its stream, event, index arrays and kernel scratch.
struct Lane {
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    uint32_t *d_idx = nullptr;          // [4][max_batch]: idx1, idx2, out slot, gate
    uint32_t *h_idx = nullptr;          // pinned staging
    void *d_accs = nullptr, *d_ext = nullptr;
    size_t accs_bytes = 0;
    std::vector<std::pair<Request *, uint32_t>> batch;
    bool busy = false;
    double t0 = 0;
};

constexpr int kLanes = 2;

struct Server {
    Context *c = nullptr;
    size_t max_batch = 0;
    uint32_t slots = 0;
    size_t W = 0;                       // words per ciphertext (n + 1)
    uint64_t *d_pool = nullptr;
    cudaStream_t up = nullptr;          // input uploads and output reads
    cudaEvent_t ev_up = nullptr;        // after the latest input upload
    Lane lane[kLanes];
    std::map<uint32_t, uint32_t> free_ranges;   // start -> length

    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request *> waiting;      // submitted, not admitted
    std::vector<Request *> active;      // admitted
    std::deque<Request *> finished;     // done, not yet polled
    uint64_t next_id = 1;
    bool stop = false;
    int fatal = FHEACC_OK;
    std::thread worker;

    // statistics
    uint64_t rounds = 0, gates_run = 0;
    double busy_s = 0, busy_since = 0;  // union of the lanes' busy intervals
    int lanes_busy = 0;

    bool alloc_range(uint32_t need, uint32_t *base)
    {
        for (auto it = free_ranges.begin(); it != free_ranges.end(); ++it) {
            if (it->second >= need) {
                *base = it->first;
                const uint32_t rest = it->second - need, start = it->first + need;
                free_ranges.erase(it);
                if (rest) free_ranges[start] = rest;
                return true;
            }
        }
        return false;
    }

    void free_range(uint32_t base, uint32_t len)
    {
        auto it = free_ranges.emplace(base, len).first;
        auto nx = std::next(it);
        if (nx != free_ranges.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_ranges.erase(nx);
        }
        if (it != free_ranges.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_ranges.erase(it);
            }
        }
    }

    // Admits waiting requests in arrival order while the pool has room
    // (caller holds mu). Returns the newly admitted ones.
    std::vector<Request *> admit_locked()
    {
        std::vector<Request *> fresh;
        while (!waiting.empty()) {
            Request *r = waiting.front();
            uint32_t base = 0;
            if (!alloc_range(r->num_inputs + r->num_gates, &base)) break;
            r->base = base;
            r->t_admit = now_s();
            waiting.pop_front();
            active.push_back(r);
            fresh.push_back(r);
        }
        return fresh;
    }

    // Copies the inputs of newly admitted requests into the pool; every
    // round launched afterwards waits for them (ev_up).
    int upload_inputs(const std::vector<Request *> &fresh)
    {
        if (fresh.empty()) return FHEACC_OK;
        for (Request *r : fresh) {
            cudaError_t e = cudaMemcpyAsync(d_pool + (size_t)r->base * W, r->inputs.data(),
                                            r->inputs.size() * sizeof(uint64_t), cudaMemcpyHostToDevice, up);
            if (e != cudaSuccess) return c->cuda_fail(e, "server input copy");
        }
        return cudaEventRecord(ev_up, up) == cudaSuccess ? FHEACC_OK : FHEACC_EIO;
    }

    bool node_ready(const Request *r, uint32_t node) const
    {
        return node < r->num_inputs || r->state[node - r->num_inputs] == 2;
    }

    // Ready gates, oldest request first, up to max_batch (caller holds mu).
    void gather_locked(std::vector<std::pair<Request *, uint32_t>> &batch)
    {
        batch.clear();
        for (Request *r : active) {
            bool blocked = false;
            for (uint32_t g = r->next_scan; g < r->num_gates && batch.size() < max_batch; g++) {
                if (r->state[g] == 0) {
                    if (node_ready(r, r->in1[g]) && node_ready(r, r->in2[g])) {
                        r->state[g] = 1;
                        batch.emplace_back(r, g);
                    } else {
                        blocked = true;
                    }
                }
                if (!blocked) r->next_scan = g + 1;   // everything below is issued or done
            }
            if (batch.size() >= max_batch) break;
        }
    }

    // One batched bootstrap of the lane's gates, reading and writing the pool
    // through the lane's index arrays.
    int launch(Lane &L)
    {
        const size_t k = L.batch.size();
        for (size_t i = 0; i < k; i++) {
            Request *r = L.batch[i].first;
            const uint32_t g = L.batch[i].second;
            L.h_idx[i] = r->base + r->in1[g];
            L.h_idx[max_batch + i] = r->base + r->in2[g];
            L.h_idx[2 * max_batch + i] = r->base + r->num_inputs + g;
            L.h_idx[3 * max_batch + i] = (uint32_t)r->type[g];
        }
        cudaError_t e = cudaStreamWaitEvent(L.st, ev_up, 0);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(L.d_idx, L.h_idx, 4 * max_batch * sizeof(uint32_t), cudaMemcpyHostToDevice, L.st);
        if (e != cudaSuccess) return c->cuda_fail(e, "server index copy");
        const uint32_t *i1 = L.d_idx, *i2 = L.d_idx + max_batch, *io = L.d_idx + 2 * max_batch;
        const int32_t *gt = reinterpret_cast<const int32_t *>(L.d_idx + 3 * max_batch);
        int rc;
        if (c->wide) {
            rc = launch_blind_rotate64_indexed(*c, d_pool, d_pool, i1, i2, gt, k, 0, (uint64_t *)L.d_accs, nullptr,
                                               (uint64_t *)L.d_ext, 0, false, L.st);
            if (!rc)
                rc = launch_lwe_keyswitch64(*c, (const uint64_t *)L.d_ext, k, true, d_pool, L.st, io, L.d_accs,
                                            L.accs_bytes);
        } else {
            rc = launch_blind_rotate32_indexed(*c, d_pool, d_pool, i1, i2, gt, k, 0, (uint32_t *)L.d_accs,
                                               (uint32_t *)L.d_ext, L.st);
            if (!rc)
                rc = launch_lwe_keyswitch32(*c, (const uint32_t *)L.d_ext, k, true, d_pool, L.st, L.d_accs,
                                            L.accs_bytes, io);
        }
        if (!rc && cudaEventRecord(L.ev, L.st) != cudaSuccess) rc = FHEACC_EIO;
        return rc;
    }

    // Marks a finished lane's gates done and completes the requests whose
    // last gate it ran (their outputs are read back here).
    int retire(Lane &L)
    {
        const double t1 = now_s();
        std::vector<Request *> complete;
        {
            std::lock_guard<std::mutex> lk(mu);
            rounds++;
            gates_run += L.batch.size();
            if (--lanes_busy == 0) busy_s += t1 - busy_since;
            for (auto &bg : L.batch) {
                bg.first->state[bg.second] = 2;
                if (++bg.first->done == bg.first->num_gates) complete.push_back(bg.first);
            }
        }
        L.busy = false;
        L.batch.clear();
        for (Request *r : complete) {
            const size_t first = (size_t)r->base + r->num_inputs + r->num_gates - r->num_outputs;
            cudaError_t e = cudaMemcpyAsync(r->out_host, d_pool + first * W,
                                            (size_t)r->num_outputs * W * sizeof(uint64_t), cudaMemcpyDeviceToHost, up);
            if (e == cudaSuccess) e = cudaStreamSynchronize(up);
            if (e != cudaSuccess) r->status = c->cuda_fail(e, "server output copy");
        }
        if (!complete.empty()) {
            std::lock_guard<std::mutex> lk(mu);
            const double t = now_s();
            for (Request *r : complete) {
                r->t_done = t;
                active.erase(std::find(active.begin(), active.end(), r));
                free_range(r->base, r->num_inputs + r->num_gates);
                finished.push_back(r);
            }
            cv_done.notify_all();
        }
        return FHEACC_OK;
    }

    // The worker: keeps up to kLanes rounds in flight. A lane whose round has
    // finished is retired (its gates done, finished requests completed); a
    // free lane takes every gate that is ready and not in flight. Requests
    // arriving meanwhile are admitted and uploaded at once, so their first
    // gates go out on the next free lane while older rounds still run.
    void run()
    {
        cudaSetDevice(c->device);
        int next_lane = 0;
        for (;;) {
            std::vector<Request *> fresh;
            bool any_active = false;
            {
                std::unique_lock<std::mutex> lk(mu);
                for (;;) {
                    fresh = admit_locked();
                    bool busy = false;
                    for (auto &L : lane) busy |= L.busy;
                    if (stop || !active.empty() || busy) break;
                    cv_work.wait(lk);
                }
                if (stop) return;
                any_active = !active.empty();
            }
            if (int rc = upload_inputs(fresh)) {
                fail_all(rc);
                return;
            }
            bool progressed = false;
            for (auto &L : lane) {
                if (!L.busy) continue;
                cudaError_t e = cudaEventQuery(L.ev);
                if (e == cudaErrorNotReady) continue;
                if (e != cudaSuccess) {
                    fail_all(c->cuda_fail(e, "server round"));
                    return;
                }
                retire(L);
                progressed = true;
            }
            for (int li = 0; li < kLanes && any_active; li++) {
                Lane &L = lane[(next_lane + li) % kLanes];
                if (L.busy) continue;
                {
                    std::lock_guard<std::mutex> lk(mu);
                    gather_locked(L.batch);
                    if (L.batch.empty()) break;
                    L.t0 = now_s();
                    if (lanes_busy++ == 0) busy_since = L.t0;
                }
                L.busy = true;
                if (int rc = launch(L)) {
                    fail_all(rc);
                    return;
                }
                next_lane = (next_lane + li + 1) % kLanes;
                progressed = true;
            }
            if (progressed) continue;
            int busy = 0;
            for (auto &L : lane) busy += L.busy;
            if (!busy) {
                // every gate of every admitted request waits on a gate that
                // is neither in flight nor done: impossible for a DAG
                bool stuck;
                {
                    std::lock_guard<std::mutex> lk(mu);
                    stuck = !active.empty();
                }
                if (stuck) {
                    fail_all(c->fail(FHEACC_EINVAL, "server: request circuit has a cycle or a dangling input"));
                    return;
                }
                continue;
            }
            if (busy == kLanes) {
                // both lanes full: block on the older round
                Lane *old = nullptr;
                for (auto &L : lane)
                    if (L.busy && (!old || L.t0 < old->t0)) old = &L;
                cudaError_t e = cudaEventSynchronize(old->ev);
                if (e != cudaSuccess) {
                    fail_all(c->cuda_fail(e, "server round"));
                    return;
                }
            } else {
                // a lane is free but nothing is ready: wait for a round to end
                // or a request to arrive
                std::unique_lock<std::mutex> lk(mu);
                cv_work.wait_for(lk, std::chrono::microseconds(100));
            }
        }
    }

    void fail_all(int rc)
    {
        std::lock_guard<std::mutex> lk(mu);
        fatal = rc ? rc : FHEACC_EIO;
        const double t = now_s();
        for (Request *r : active) {
            r->status = fatal;
            r->t_done = t;
            finished.push_back(r);
        }
        for (Request *r : waiting) {
            r->status = fatal;
            r->t_done = t;
            finished.push_back(r);
        }
        active.clear();
        waiting.clear();
        cv_done.notify_all();
    }
};

// Frees everything a server holds (its worker has stopped); the device is current.
static void server_release(Server *s)
{
    for (auto &L : s->lane)
        if (L.st) cudaStreamSynchronize(L.st);
    if (s->up) cudaStreamSynchronize(s->up);
    for (Request *r : s->waiting) delete r;
    for (Request *r : s->active) delete r;
    for (Request *r : s->finished) delete r;
    for (auto &L : s->lane) {
        cudaFree(L.d_idx);
        cudaFreeHost(L.h_idx);
        cudaFree(L.d_accs);
        cudaFree(L.d_ext);
        if (L.ev) cudaEventDestroy(L.ev);
        if (L.st) cudaStreamDestroy(L.st);
    }
    cudaFree(s->d_pool);
    if (s->ev_up) cudaEventDestroy(s->ev_up);
    if (s->up) cudaStreamDestroy(s->up);
    delete s;
}

}  // namespace fheacc

using namespace fheacc;

extern "C" {

int fheacc_server_create(fheacc_ctx *ctx, size_t max_batch, size_t pool_ciphertexts, fheacc_server **out)
{
    if (!ctx || !out || max_batch == 0 || max_batch > (1u << 24) || pool_ciphertexts > 0xFFFFFFF0u)
        return FHEACC_EINVAL;
    Context &c = *reinterpret_cast<Context *>(ctx);
    if (c.wide ? (!c.d_btkey64 || !c.d_kskey64) : (!c.d_btkey || !c.d_kskey))
        return c.fail(FHEACC_ENOKEY, "server: keys must be uploaded first");
    DeviceGuard guard(c.device);
    Server *s = new Server();
    s->c = &c;
    s->max_batch = max_batch;
    s->W = (size_t)c.p.n + 1;
    const size_t ct_bytes = s->W * sizeof(uint64_t);
    const size_t lane_bytes = 4 * max_batch * sizeof(uint32_t) + bootstrap_accs_bytes(c, max_batch) +
                              bootstrap_extract_bytes(c, max_batch);
    if (pool_ciphertexts == 0) {
        // a quarter of the device memory free now (after the lanes' scratch),
        // at most 32 GiB
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess || free_b < kLanes * lane_bytes) {
            cudaGetLastError();
            delete s;
            return c.fail(FHEACC_ENOMEM, "server: no free device memory for the pool");
        }
        const size_t pool_b = std::min<size_t>((free_b - kLanes * lane_bytes) / 4, (size_t)32 << 30);
        pool_ciphertexts = std::min<size_t>(pool_b / ct_bytes, 0xFFFFFFF0u);
        if (pool_ciphertexts == 0) {
            delete s;
            return c.fail(FHEACC_ENOMEM, "server: no free device memory for the pool");
        }
    }
    s->slots = (uint32_t)pool_ciphertexts;
    cudaError_t e = cudaMalloc(&s->d_pool, (size_t)s->slots * ct_bytes);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->up, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev_up, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(s->ev_up, s->up);
    for (auto &L : s->lane) {
        L.accs_bytes = bootstrap_accs_bytes(c, max_batch);
        if (e == cudaSuccess) e = cudaMalloc(&L.d_idx, 4 * max_batch * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMallocHost(&L.h_idx, 4 * max_batch * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMalloc(&L.d_accs, L.accs_bytes);
        if (e == cudaSuccess) e = cudaMalloc(&L.d_ext, bootstrap_extract_bytes(c, max_batch));
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&L.st, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&L.ev, cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        server_release(s);
        return c.fail(FHEACC_ENOMEM, std::string("server allocation: ") + cudaGetErrorString(e));
    }
    s->free_ranges[0] = s->slots;
    s->worker = std::thread([s] { s->run(); });
    *out = reinterpret_cast<fheacc_server *>(s);
    return FHEACC_OK;
}

int fheacc_server_submit(fheacc_server *srv, const uint64_t *inputs, uint32_t num_inputs, const int32_t *gate_types,
                         const uint32_t *in1, const uint32_t *in2, uint32_t num_gates, uint32_t num_outputs,
                         uint64_t *out, uint64_t *request_id)
{
    if (!srv || !inputs || num_inputs == 0 || num_gates == 0 || !gate_types || !in1 || !in2 || !out ||
        num_outputs == 0 || num_outputs > num_gates)
        return FHEACC_EINVAL;
    Server &s = *reinterpret_cast<Server *>(srv);
    if ((uint64_t)num_inputs + num_gates > s.slots) return s.c->fail(FHEACC_EINVAL, "server: request larger than the pool");
    for (uint32_t g = 0; g < num_gates; g++) {
        const uint32_t node = num_inputs + g;
        if (in1[g] >= node || in2[g] >= node || in1[g] == in2[g] || gate_types[g] < 0 || gate_types[g] > 5)
            return s.c->fail(FHEACC_EINVAL, "server: gate inputs must be two distinct earlier nodes, gate code 0..5");
    }
    Request *r = new Request();
    r->num_inputs = num_inputs;
    r->num_gates = num_gates;
    r->num_outputs = num_outputs;
    r->type.assign(gate_types, gate_types + num_gates);
    r->in1.assign(in1, in1 + num_gates);
    r->in2.assign(in2, in2 + num_gates);
    r->inputs.assign(inputs, inputs + (size_t)num_inputs * s.W);
    r->out_host = out;
    r->state.assign(num_gates, 0);
    r->t_submit = now_s();
    {
        std::lock_guard<std::mutex> lk(s.mu);
        if (s.fatal) {
            delete r;
            return s.fatal;
        }
        r->id = s.next_id++;
        s.waiting.push_back(r);
    }
    s.cv_work.notify_one();
    if (request_id) *request_id = r->id;
    return FHEACC_OK;
}

int fheacc_server_poll(fheacc_server *srv, fheacc_request_done *done, size_t max, size_t *n_done, uint32_t timeout_ms)
{
    if (!srv || !done || !n_done) return FHEACC_EINVAL;
    Server &s = *reinterpret_cast<Server *>(srv);
    std::unique_lock<std::mutex> lk(s.mu);
    if (s.finished.empty() && timeout_ms)
        s.cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return !s.finished.empty(); });
    size_t k = 0;
    while (k < max && !s.finished.empty()) {
        Request *r = s.finished.front();
        s.finished.pop_front();
        done[k].request_id = r->id;
        done[k].status = r->status;
        done[k].queue_ms = (r->t_admit > 0 ? r->t_admit - r->t_submit : r->t_done - r->t_submit) * 1e3;
        done[k].latency_ms = (r->t_done - r->t_submit) * 1e3;
        delete r;
        k++;
    }
    *n_done = k;
    return FHEACC_OK;
}

int fheacc_server_stats(fheacc_server *srv, fheacc_server_stats_t *st)
{
    if (!srv || !st) return FHEACC_EINVAL;
    Server &s = *reinterpret_cast<Server *>(srv);
    std::lock_guard<std::mutex> lk(s.mu);
    st->rounds = s.rounds;
    st->gates = s.gates_run;
    st->busy_s = s.busy_s;
    st->waiting = s.waiting.size();
    st->active = s.active.size();
    uint64_t free_slots = 0;
    for (auto &kv : s.free_ranges) free_slots += kv.second;
    st->free_slots = free_slots;
    st->pool_slots = s.slots;
    st->lanes = kLanes;
    return FHEACC_OK;
}

int fheacc_server_destroy(fheacc_server *srv)
{
    if (!srv) return FHEACC_OK;
    Server *s = reinterpret_cast<Server *>(srv);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    DeviceGuard guard(s->c->device);
    server_release(s);
    return FHEACC_OK;
}

}  // extern "C"
