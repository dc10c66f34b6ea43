"""Gate-bootstrapping throughput on GB300.

One step = one batched gate-bootstrapping pass over a fixed synthetic batch:
4096 independent NAND gates with the n=500, N=1024, Q=134215681 (uint32),
BG=2^7 x4 parameter set, keys and inputs generated from fixed seeds.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line. `value` is bootstraps/s with inputs resident in HBM,
timed with CUDA events on the launching stream (L2 flushed between steps);
`e2e` is the same metric through the host-buffer C-ABI call fheacc_bootstrap
(host->device copies, the kernels and device->host copies inside the timed
region). `--impl reference` times the CPU restatement of the reference's
eval_bootstrap (oracle/) on all host cores on the same workload.
Under torchrun every rank bootstraps its own batch on its own GPU (the gates
are independent: no collective on the data path) and rank 0 reports the
aggregate over the max-over-ranks time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

METRIC = "gate bootstraps/sec on 1 GB300 (batched persistent vs plain per-gate launch, bit-exact); p99 ms"
SEEDS = dict(lwe_sk=1, rlwe_sk=2, btkey=3, kskey=4, enc=5)
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
TRAFFIC_FILE = os.path.join(ROOT, "profiles", "traffic.json")


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    def __init__(self, use_cuda):
        self.ws, self.rank, self.local = dist_env()
        self.pg = None
        if self.ws > 1:
            import torch.distributed as td
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            td.init_process_group("nccl" if use_cuda else "gloo")
            self.td = td

    def barrier(self):
        if self.ws > 1:
            self.td.barrier()

    def max(self, x):
        if self.ws == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.td.destroy_process_group()


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = max(smax, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def steps_of(c1, c2, gates, P):
    """Exact number of RLWE x RGSW steps of each gate (RLWE.cpp:754-767)."""
    q = P.q
    a1 = c1[:, :P.n].astype(np.int64)
    a2 = c2[:, :P.n].astype(np.int64)
    x2 = ((gates == 4) | (gates == 5))[:, None]
    a = np.where(x2, 2 * (a1 - a2), a1 + a2) % q
    nega = (q - a) % q
    steps = np.zeros(c1.shape[0], dtype=np.int64)
    for _ in range(P.digitR):
        steps += (nega % P.Br != 0).sum(axis=1)
        nega //= P.Br
    return steps


class KeyCache:
    """One key set (secret keys, bootstrap and key-switch keys, a context with
    both uploaded) per preset, made once and shared by the blocks of a run."""

    def __init__(self, F, device=0):
        self.F, self.device, self.sets = F, device, {}

    def get(self, preset):
        if preset not in self.sets:
            F = self.F
            P = F.params_preset(preset)
            lsk = F.LWE_secretkey(P, SEEDS["lwe_sk"])
            rsk = F.RLWE_secretkey(P, SEEDS["rlwe_sk"])
            bt = F.bootstrap_key(P, SEEDS["btkey"], lsk, rsk)
            ks = F.keyswitch_key(P, SEEDS["kskey"], rsk, lsk)
            ctx = F.Context(P, self.device)
            ctx.upload_bootstrap_key(bt)
            ctx.upload_keyswitch_key(ks)
            self.sets[preset] = dict(P=P, lsk=lsk, rsk=rsk, bt=bt, ks=ks, ctx=ctx)
        return self.sets[preset]

    def close(self):
        for s in self.sets.values():
            s["ctx"].close()
        self.sets = {}


def make_inputs(F, P, batch, rank):
    lsk = F.LWE_secretkey(P, SEEDS["lwe_sk"])
    rsk = F.RLWE_secretkey(P, SEEDS["rlwe_sk"])
    rng = np.random.default_rng(1000 + rank)
    x = rng.integers(0, 2, batch).astype(np.uint8)
    y = rng.integers(0, 2, batch).astype(np.uint8)
    c = F.LWE_encrypt(P, SEEDS["enc"] + 7919 * rank, lsk, np.concatenate([x, y]))
    gates = np.full(batch, F.NAND, dtype=np.int32)
    return lsk, rsk, x, y, c[:batch].copy(), c[batch:].copy(), gates


def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def run_reference(args):
    """CPU restatement of eval_bootstrap (oracle/), all host cores. Keys,
    inputs and parameters come from the oracle alone (its own seeded key
    generation): this arm loads no product library."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from oracle_lib import Oracle
    ora = Oracle.preset(args.preset)
    P = ora.p
    cores = cpu_cores()
    lsk, rsk, bt, ks = ora.keygen(SEEDS["lwe_sk"], threads=cores)
    rng = np.random.default_rng(1000)
    x = rng.integers(0, 2, args.batch).astype(np.uint8)
    y = rng.integers(0, 2, args.batch).astype(np.uint8)
    c = ora.lwe_encrypt(SEEDS["enc"], lsk, np.concatenate([x, y]))
    c1, c2 = c[:args.batch].copy(), c[args.batch:].copy()
    gates = np.full(args.batch, 3, dtype=np.int32)   # NAND (params.h:107)
    per_step = args.cpu_sample or (2 if P.N == 1024 else 1) * cores
    times = []
    for s in range(args.warmup + args.steps):
        lo = (s * per_step) % max(args.batch - per_step, 1)
        t0 = time.perf_counter()
        out, failed = ora.eval_bootstrap_batch(c1[lo:lo + per_step], c2[lo:lo + per_step], gates[lo:lo + per_step],
                                               bt, ks, threads=cores)
        dt = time.perf_counter() - t0
        assert failed == 0
        dec = np.array([ora.lwe_decrypt(lsk, o) for o in out], dtype=np.uint8)
        assert np.array_equal(dec, 1 - (x[lo:lo + per_step] & y[lo:lo + per_step])), "oracle NAND decrypts wrong"
        if s >= args.warmup:
            times.append(dt)
    value = per_step / statistics.mean(times)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "bootstraps/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": config_of(param_view(P), args.batch),
        "cpu_baseline": {"value": value, "unit": "bootstraps/s", "cores": cores, "kind": "port",
                         "sample": "%d gates per step of the %d-gate batch, oracle eval_bootstrap "
                                   "(C restatement of RLWE.cpp:726-786) on %d threads; keys from the oracle's own "
                                   "generator" % (per_step, args.batch, cores)},
        "e2e": {"value": value, "unit": "bootstraps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def param_view(p):
    """The fields config_of reads, from an oracle parameter set."""
    class V:
        pass
    v = V()
    v.n, v.q, v.N, v.Q, v.BG_bits, v.digitG = p.n, p.q, p.N, p.Q, p.BGbits, p.digitG
    v.Br, v.digitR, v.Bks, v.digitKS = p.Br, p.digitR, p.Bks, p.digitKS
    return v


def profile_case(preset=0, gates=912, n=64):
    """The case the committed ncu section captures use: the bench parameter
    set with n = 64 (same per-step work), 912 random gates (6 per SM: the
    3-pipeline shape of the 32-bit kernel, one wave of the 64-bit grid), two
    batched launches, outputs checked by decryption. gates = 1, n = 500: a
    lone gate of the bench set (the latency form of the 32-bit kernel)."""
    import torch
    import __graft_entry__
    __graft_entry__.build_product()
    import importlib
    F = importlib.import_module("3rd_gen_fhe_acc_gb300")
    P = F.params_preset(preset)
    P.n = n
    F.derive(P)
    lsk = F.LWE_secretkey(P, 1)
    rsk = F.RLWE_secretkey(P, 2)
    ctx = F.Context(P, 0)
    ctx.upload_bootstrap_key(F.bootstrap_key(P, 3, lsk, rsk))
    ctx.upload_keyswitch_key(F.keyswitch_key(P, 4, rsk, lsk))
    B = gates
    rng = np.random.default_rng(0)
    bits = rng.integers(0, 2, 2 * B).astype(np.uint8)
    c = F.LWE_encrypt(P, 9, lsk, bits)
    g = rng.integers(0, 6, B).astype(np.int32)
    d1 = torch.from_numpy(c[:B].view(np.int64)).cuda()
    d2 = torch.from_numpy(c[B:].view(np.int64)).cuda()
    dg = torch.from_numpy(g).cuda()
    out = torch.zeros_like(d1)
    for _ in range(2):
        ctx.bootstrap_async(d1.data_ptr(), d2.data_ptr(), dg.data_ptr(), B, out.data_ptr())
    torch.cuda.synchronize()
    dec = F.LWE_decrypt(P, lsk, out.cpu().numpy().view(np.uint64))
    truth = np.array([F.gate_truth(int(a), x, y) for a, x, y in zip(g, bits[:B], bits[B:])], dtype=np.uint8)
    ok = int((dec == truth).sum())
    print("profile case: %d/%d gates decrypt correctly" % (ok, B))
    ctx.close()
    return 0 if ok == B else 1


def run_serving(F, ctx, P, lsk, rate, duration, kmax=256, seed=7, max_batch=2048, pool=1 << 20):
    """Poisson stream of PSI equality queries (a 32-bit client item against
    k ~ U[1, kmax] encrypted server items: 32 XNOR + a 31-gate AND tree per
    item) at `rate` bootstraps/s for `duration` seconds through the
    continuous-batching server; returns latency percentiles and throughput."""
    rng = np.random.default_rng(seed)
    mean_gates = 63 * (kmax + 1) / 2
    req_rate = rate / mean_gates
    # pre-generate the requests (encryption is not part of the served path)
    arrivals, reqs = [], []
    t = 0.0
    while True:
        t += rng.exponential(1.0 / req_rate)
        if t > duration:
            break
        k = int(rng.integers(1, kmax + 1))
        bits = rng.integers(0, 2, 32 * (k + 1)).astype(np.uint8)
        arrivals.append(t)
        reqs.append((F.LWE_encrypt(P, 50_000 + len(reqs), lsk, bits), F.psi_equality_circuit(k)))
    if not reqs:
        return None
    srv = F.Server(ctx, max_batch=max_batch, pool_ciphertexts=pool)
    lat, queue = [], []
    done_gates = 0
    gates_of = {}
    t0 = time.perf_counter()

    def feeder():
        for ta, (ct, circ) in zip(arrivals, reqs):
            d = ta - (time.perf_counter() - t0)
            if d > 0:
                time.sleep(d)
            rid, _ = srv.submit(ct, *circ)
            gates_of[rid] = len(circ[0])

    th = threading.Thread(target=feeder)
    th.start()
    while len(lat) < len(reqs):
        for rid, status, q_ms, l_ms, out in srv.poll(timeout_ms=100):
            assert status == 0
            lat.append(l_ms)
            queue.append(q_ms)
            done_gates += gates_of.get(rid, 0)
        if time.perf_counter() - t0 > duration + 600:
            break
    elapsed = time.perf_counter() - t0
    th.join()
    st = srv.stats()
    srv.close()
    return {"offered_bootstraps_per_s": rate, "requests": len(lat), "items_per_request": "U[1,%d]" % kmax,
            "max_batch": max_batch, "gates": int(st["gates"]), "rounds": int(st["rounds"]),
            "throughput_bootstraps_per_s": st["gates"] / elapsed, "duration_s": elapsed,
            "latency_ms_p50": float(np.percentile(lat, 50)), "latency_ms_p99": float(np.percentile(lat, 99)),
            "queue_ms_p99": float(np.percentile(queue, 99)), "gpu_busy_frac": st["busy_s"] / elapsed}


def run_mixed(args, cache=None):
    """Uneven batching (one CUDA-graph launch per step): requests of geometric
    size (mean 64, from a seed) until 3000 N=1024 and 700 N=2048 gates, the two
    parameter sets as two contexts, each autotuned for its batch, both batches
    captured into one graph. Returns the line (printed when run alone)."""
    import torch
    import __graft_entry__
    __graft_entry__.build_product()
    import importlib
    F = importlib.import_module("3rd_gen_fhe_acc_gb300")
    torch.cuda.set_device(0)
    own = cache is None
    cache = cache or KeyCache(F)
    rng = np.random.default_rng(args.mixed_seed)
    sets = []
    for preset, total in ((0, args.mixed_narrow), (1, args.mixed_wide)):
        counts = []
        while sum(counts) < total:
            counts.append(int(min(rng.geometric(1.0 / 64), total - sum(counts))))
        sets.append({"preset": preset, "P": F.params_preset(preset), "counts": counts, "total": total})
    arrival = [(si, ri) for si, st_ in enumerate(sets) for ri in range(len(st_["counts"]))]
    rng.shuffle(arrival)
    stream = torch.cuda.current_stream()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    t_setup = time.perf_counter()
    for si, S in enumerate(sets):
        P, B = S["P"], S["total"]
        # the set's requests laid out in arrival order
        order = [ri for (sj, ri) in arrival if sj == si]
        offs, off = {}, 0
        for ri in order:
            offs[ri] = off
            off += S["counts"][ri]
        S["offsets"] = offs
        K = cache.get(S["preset"])
        lsk = K["lsk"]
        x = rng.integers(0, 2, B).astype(np.uint8)
        y = rng.integers(0, 2, B).astype(np.uint8)
        g = rng.integers(0, 6, B).astype(np.int32)
        c = F.LWE_encrypt(P, SEEDS["enc"] + 31 * si, lsk, np.concatenate([x, y]))
        S.update(lsk=lsk, x=x, y=y, g=g, c1=c[:B].copy(), c2=c[B:].copy(),
                 truth=np.array([F.gate_truth(int(a), b, d) for a, b, d in zip(g, x, y)], dtype=np.uint8))
        S["bt"], S["ks"], S["ctx"] = K["bt"], K["ks"], K["ctx"]
        S["d1"] = torch.from_numpy(S["c1"].view(np.int64)).cuda()
        S["d2"] = torch.from_numpy(S["c2"].view(np.int64)).cuda()
        S["dg"] = torch.from_numpy(g).cuda()
        S["dout"] = torch.zeros_like(S["d1"])
    setup_s = time.perf_counter() - t_setup

    # one launch per set, untuned and tuned: reference outputs and per-set times
    def alone(S, reps=3):
        ts = []
        for r in range(reps):
            flush.fill_(1)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            S["ctx"].bootstrap_async(S["d1"].data_ptr(), S["d2"].data_ptr(), S["dg"].data_ptr(), S["total"],
                                     S["dout"].data_ptr(), 0, stream.cuda_stream)
            e1.record(stream)
            torch.cuda.synchronize()
            if r:
                ts.append(e0.elapsed_time(e1))
        return min(ts)

    for S in sets:
        S["untuned_ms"] = alone(S)
        S["ref_out"] = S["dout"].cpu().numpy().view(np.uint64).copy()
        S["trials"] = S["ctx"].autotune(S["total"])
        S["tuned_ms"] = alone(S)
        S["tuned_same"] = np.array_equal(S["dout"].cpu().numpy().view(np.uint64), S["ref_out"])
        best = min(S["trials"], key=lambda t: t["ms"])
        S["best"] = {k: best[k] for k in ("regs_for_3", "ctas_per_sm", "group", "window", "pipes")}

    graph = F.Graph()
    for S in sets:
        graph.add(S["ctx"], S["d1"].data_ptr(), S["d2"].data_ptr(), S["dg"].data_ptr(), S["total"],
                  S["dout"].data_ptr())
    # the same batches as concurrent branches (reported beside the serial graph)
    cgraph = F.Graph(concurrent=True)
    for S in sets:
        cgraph.add(S["ctx"], S["d1"].data_ptr(), S["d2"].data_ptr(), S["dg"].data_ptr(), S["total"],
                   S["dout"].data_ptr())
    conc_ms = []
    for r in range(3):
        flush.fill_(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        cgraph.launch(stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        if r:
            conc_ms.append(e0.elapsed_time(e1))
    conc_same = all(np.array_equal(S["dout"].cpu().numpy().view(np.uint64), S["ref_out"]) for S in sets)
    cgraph.close()
    for S in sets:
        S["dout"].zero_()
    n0 = sum(S["ctx"].kernel_launches() for S in sets)
    for _ in range(args.warmup):
        flush.fill_(1)
        graph.launch(stream.cuda_stream)
    torch.cuda.synchronize()
    # the graph is captured at its first launch: its kernels, launched by every replay
    per_replay = sum(S["ctx"].kernel_launches() for S in sets) - n0
    outs_ok = all(np.array_equal(S["dout"].cpu().numpy().view(np.uint64), S["ref_out"]) for S in sets)
    clocks = ClockSampler(0)
    clocks.start()
    step_ms = []
    for _ in range(args.steps):
        flush.fill_(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        graph.launch(stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        step_ms.append(e0.elapsed_time(e1))
    clk = clocks.stop()
    total = sum(S["total"] for S in sets)
    value = total * args.steps / (sum(step_ms) / 1e3)

    # e2e: pinned host inputs -> device, graph, outputs -> host, every step
    pins = []
    for S in sets:
        pins.append([torch.from_numpy(S["c1"].view(np.int64)).pin_memory(),
                     torch.from_numpy(S["c2"].view(np.int64)).pin_memory(),
                     torch.from_numpy(S["g"]).pin_memory(), torch.zeros_like(S["dout"], device="cpu").pin_memory()])
    h2d = sum(p[0].numel() * 8 + p[1].numel() * 8 + p[2].numel() * 4 for p in pins)
    d2h = sum(p[3].numel() * 8 for p in pins)
    e2e = []
    for s_ in range(args.warmup + args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for S, p in zip(sets, pins):
            S["d1"].copy_(p[0], non_blocking=True)
            S["d2"].copy_(p[1], non_blocking=True)
            S["dg"].copy_(p[2], non_blocking=True)
        graph.launch(stream.cuda_stream)
        for S, p in zip(sets, pins):
            p[3].copy_(S["dout"], non_blocking=True)
        torch.cuda.synchronize()
        if s_ >= args.warmup:
            e2e.append(time.perf_counter() - t0)
    e2e_value = total * args.steps / sum(e2e)
    dec_ok = {}
    per_request_ok = True
    for S, p in zip(sets, pins):
        o = p[3].numpy().view(np.uint64)
        dec = F.LWE_decrypt(S["P"], S["lsk"], o)
        dec_ok["N=%d" % S["P"].N] = "%d/%d" % (int((dec == S["truth"]).sum()), S["total"])
        per_request_ok &= np.array_equal(o, S["ref_out"])
        for ri, off in S["offsets"].items():   # every request's slice
            k = S["counts"][ri]
            per_request_ok &= bool((dec[off:off + k] == S["truth"][off:off + k]).all())

    cpu = None
    if not args.no_cpu:
        import __graft_entry__ as ge
        ge._build_oracle()
        from oracle_lib import Oracle
        cores = cpu_cores()
        rates, samples = [], []
        for S in sets:
            ora = Oracle.from_params(S["P"])
            ns = (8 if S["P"].N == 1024 else 1) * cores
            t0 = time.perf_counter()
            co, failed = ora.eval_bootstrap_batch(S["c1"][:ns], S["c2"][:ns], S["g"][:ns], S["bt"], S["ks"],
                                                  threads=cores)
            dt = time.perf_counter() - t0
            rates.append(ns / dt)
            samples.append("%d N=%d gates in %.1f s (%s)" % (ns, S["P"].N, dt, "bit-exact" if np.array_equal(
                co, S["ref_out"][:ns]) and failed == 0 else "MISMATCH"))
        cpu_value = total / sum(S["total"] / r for S, r in zip(sets, rates))
        cpu = {"value": cpu_value, "unit": "bootstraps/s", "cores": cores, "kind": "port",
               "sample": "oracle eval_bootstrap (C restatement of RLWE.cpp:726-786) on %d threads: %s; mixed rate "
                         "= harmonic combination over the batch" % (cores, "; ".join(samples))}
    line = {
        "metric": "gate bootstraps/sec on 1 GB300, uneven batch in one CUDA-graph launch (bit-exact)",
        "value": value, "unit": "bootstraps/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": statistics.mean(step_ms), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32+u64", "data": "synthetic",
        "config": {"workload": "uneven batch: %d N=1024 (n=500, Q<2^27, BG=2^7 x4) + %d N=2048 (n=630, Q<2^54, "
                               "BG=2^9 x6) gate bootstraps from %d requests of geometric size (mean 64), seed %d, "
                               "one CUDA-graph launch" % (sets[0]["total"], sets[1]["total"],
                                                          sum(len(S["counts"]) for S in sets), args.mixed_seed),
                   "requests": {"N=%d" % S["P"].N: len(S["counts"]) for S in sets},
                   "l2": "flushed between timed steps (write of a 512 MiB buffer)",
                   "parallelism": "one graph per GPU; the two parameter sets in order on one branch"},
        "e2e": {"value": e2e_value, "unit": "bootstraps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": 1e3 * statistics.mean(e2e)},
        "per_set": {"N=%d" % S["P"].N: {"gates": S["total"], "alone_untuned_ms": S["untuned_ms"],
                                         "alone_tuned_ms": S["tuned_ms"], "autotuned": S["best"],
                                         "trials": len(S["trials"])} for S in sets},
        "graph_vs_sum_of_alone": sum(S["tuned_ms"] for S in sets) / statistics.mean(step_ms),
        "concurrent_branches": {"ms_per_step": min(conc_ms), "bitexact": bool(conc_same),
                                "note": "the two sets as concurrent graph branches; the persistent grids then "
                                        "share SMs unevenly"},
        "cpu_baseline": cpu, "clocks": clk, "gpu_launches": per_replay * args.steps,
        "checks": {"decrypt_ok": dec_ok, "graph_equals_separate_launches": bool(outs_ok),
                   "tuned_equals_untuned": all(S["tuned_same"] for S in sets),
                   "every_request_decrypts": bool(per_request_ok), "setup_s": setup_s},
    }
    for S in sets:   # the contexts go back to their defaults
        for opt, v in ((F.OPT_BR_REGS_FOR_3, -1), (F.OPT_BR_CTAS_PER_SM, 0), (F.OPT_BR_GROUP, 0),
                       (F.OPT_BR_WINDOW, -1), (F.OPT_BR_PIPES, 0)):
            S["ctx"].set_option(opt, v)
    if own:
        print(json.dumps(line))
        cache.close()
    return line


def run_psi(args, cache=None):
    """One PSI query of the reference's PSI test (test.cpp:1510-1606) per step,
    at N = 2048 (the 64-bit set): homo_expand of digitG packed RLWEs into N
    RGSWs (app.cpp:78-96), a CMUX tree selecting one of 2^(18 - log2 N) = 128
    database RLWEs (RLWE.cpp:788-793), and an RLWE blind rotation of the
    selected entry (RLWE.cpp:824-838). Plaintexts are made with the library's
    own NTT; the query sets every odd bit, so the result decrypts to ones at
    coefficients 1366..1451."""
    import torch
    import __graft_entry__
    __graft_entry__.build_product()
    import importlib
    F = importlib.import_module("3rd_gen_fhe_acc_gb300")
    torch.cuda.set_device(0)
    P = F.params_preset(1)
    F.derive(P)
    N, Q, dG, logN = P.N, P.Q, P.digitG, 11
    rw, gw = 2 * N, dG * 4 * N
    t_setup = time.perf_counter()
    own = cache is None
    if own:
        rsk = F.RLWE_secretkey(P, 12)
        ctx = F.Context(P, 0)
    else:
        K = cache.get(1)
        rsk, ctx = K["rsk"], K["ctx"]
    subs = F.substitute_key(P, 15, rsk)
    ctx.upload_subs_key(subs)
    stream = torch.cuda.current_stream()
    st = stream.cuda_stream

    def ntt_host(polys, inverse=False):
        d = torch.from_numpy(np.ascontiguousarray(polys, dtype=np.uint64).view(np.int64)).cuda()
        (ctx.ntt_inverse if inverse else ctx.ntt_forward)(d.data_ptr(), d.numel() // N, st)
        torch.cuda.synchronize()
        return d.cpu().numpy().view(np.uint64)

    s_time = ntt_host(rsk, inverse=True)
    enc_neg_s = F.RGSW_encrypt(P, 41, rsk, ntt_host((Q - s_time) % Q))
    iN = pow(N, Q - 2, Q)
    packed, pow_bg = [], 1
    for i in range(dG):
        m = np.zeros(N, dtype=np.uint64)
        m[1::2] = pow_bg * iN % Q
        packed.append(F.RLWE_encrypt(P, 100 + i, rsk, ntt_host(m)))
        pow_bg = pow_bg * (1 << P.BG_bits) % Q
    packed = np.concatenate(packed)
    entries = 1 << (18 - logN)
    db = []
    for i in range(entries):
        m = np.zeros(N, dtype=np.uint64)
        m[:i + 1] = Q // 2
        db.append(F.RLWE_encrypt(P, 1000 + i, rsk, ntt_host(m)))
    db = np.concatenate(db)
    setup_s = time.perf_counter() - t_setup
    dv = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint64).view(np.int64)).cuda()
    d_packed, d_enc, d_db = dv(packed), dv(enc_neg_s), dv(db)
    rgsw = torch.zeros(N * gw, dtype=torch.int64, device="cuda")
    bufs = [torch.zeros(entries // 2 * rw, dtype=torch.int64, device="cuda") for _ in range(2)]
    out = torch.zeros(rw, dtype=torch.int64, device="cuda")
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")

    def query(ev=None):
        if ev: ev[0].record(stream)
        ctx.homo_expand(d_packed.data_ptr(), d_enc.data_ptr(), rgsw.data_ptr(), st)
        if ev: ev[1].record(stream)
        src, count, level = d_db, entries, logN
        while count > 1:   # v[k] = CMUX(v[2k], v[2k+1], RGSW[level])
            dst = bufs[level & 1]
            ctx.CMUX(src.data_ptr(), src.data_ptr() + 8 * rw, rgsw.data_ptr() + 8 * gw * level, dst.data_ptr(),
                     count // 2, in_stride=2 * rw, stream=st)
            src, count, level = dst, count // 2, level + 1
        if ev: ev[2].record(stream)
        ctx.blind_rotate_RLWE(src.data_ptr(), rgsw.data_ptr(), False, out.data_ptr(), 1, stream=st)
        if ev: ev[3].record(stream)

    want = np.zeros(N, dtype=np.uint8)
    want[1366:1452] = 1

    def decodes(o):
        phase = F.RLWE_phase(P, rsk, o)
        return np.array_equal(((2 * phase.astype(object) + Q // 2) // Q % 2).astype(np.uint8), want)

    for _ in range(args.warmup):
        flush.fill_(1)
        query()
    torch.cuda.synchronize()
    first_out = out.cpu().numpy().view(np.uint64).copy()
    clocks = ClockSampler(0)
    clocks.start()
    phases = []
    n0 = ctx.kernel_launches()
    for _ in range(args.steps):
        flush.fill_(1)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        torch.cuda.synchronize()
        query(ev)
        torch.cuda.synchronize()
        phases.append([ev[i].elapsed_time(ev[i + 1]) for i in range(3)])
    clk = clocks.stop()
    launches = ctx.kernel_launches() - n0
    step_ms = [sum(ph) for ph in phases]
    value = args.steps / (sum(step_ms) / 1e3)
    repeat_ok = np.array_equal(out.cpu().numpy().view(np.uint64), first_out)

    # e2e: the query's packed RLWEs in from pinned host memory, the result out
    h_packed = torch.from_numpy(packed.view(np.int64)).pin_memory()
    h_out = torch.zeros(rw, dtype=torch.int64).pin_memory()
    e2e = []
    for s_ in range(args.warmup + args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d_packed.copy_(h_packed, non_blocking=True)
        query()
        h_out.copy_(out, non_blocking=True)
        torch.cuda.synchronize()
        if s_ >= args.warmup:
            e2e.append(time.perf_counter() - t0)
    e2e_ok = decodes(h_out.numpy().view(np.uint64))

    # integer roofline: 64-bit modular multiplies of the query, the reference's
    # algorithm (an N = 2048 NTT is N/2 log2 N butterflies, an inverse NTT that
    # plus N scalings): per expand item (one RLWE of one level) the inverse
    # NTTs of a and b, digitKS_R + 1 forward NTTs, 2 digitKS_R N key products
    # and 2N for the rotation; per RLWE x RGSW 210,944 as in the bootstrap
    L = P.digitKS_R
    ntt = N // 2 * logN
    mult = 2 * (ntt + N) + 2 * dG * ntt + 4 * dG * N   # 210,944
    expand_item = 2 * (ntt + N) + (L + 1) * ntt + 2 * L * N + 2 * N
    items = dG * (N - 1)
    n_mult = dG * N + (entries - 1) + logN
    work = items * expand_item + n_mult * mult + logN * 2 * N
    imad = ctx.measure_imad_rate()
    slots = 16
    peak = imad / slots
    achieved = work / (statistics.mean(step_ms) / 1e3)
    roofline = {"bound": "int", "achieved": achieved / 1e9, "peak": peak / 1e9, "unit": "G modmul/s",
                "frac": achieved / peak, "traffic": None, "kernel": "whole query",
                "work": "%d expand items x %d + %d RLWE x RGSW x %d + %d rotation multiplies = %.3g 64-bit modular "
                        "multiplies per query" % (items, expand_item, n_mult, mult, logN * 2 * N, work),
                "peak_source": "IMAD rate measured in this run (%.1f T lane-op/s) / %d IMAD issue slots per 64-bit "
                               "Shoup modular multiply" % (imad / 1e12, slots)}

    cpu = None
    if not args.no_cpu:
        import __graft_entry__ as ge
        ge._build_oracle()
        from oracle_lib import Oracle
        ora = Oracle.from_params(P)
        t0 = time.perf_counter()
        r_exp = ora.expand_rlwe(packed[:rw], subs)
        t_exp = time.perf_counter() - t0
        sample_m = 8
        t0 = time.perf_counter()
        for k in range(sample_m):
            ora.rlwe_mult_rgsw(r_exp[k], enc_neg_s)
        t_mult = (time.perf_counter() - t0) / sample_m
        t0 = time.perf_counter()
        for k in range(sample_m):
            ora.cmux(db[k * rw:(k + 1) * rw], db[(k + 1) * rw:(k + 2) * rw], enc_neg_s)
        t_cmux = (time.perf_counter() - t0) / sample_m
        cpu_query_s = dG * (t_exp + N * t_mult) + (entries - 1 + logN) * t_cmux
        cpu = {"value": 1.0 / cpu_query_s, "unit": "PSI queries/s", "cores": 1, "kind": "port",
               "sample": "oracle (C restatement of app.cpp:26-96, RLWE.cpp:642-704,788-838) on one thread: one "
                         "expand_RLWE %.1f s, RLWE x RGSW %.1f ms and CMUX %.1f ms (means of %d); a query = %d "
                         "expand_RLWE + %d RLWE x RGSW + %d CMUX = %.0f s" % (
                             t_exp, 1e3 * t_mult, 1e3 * t_cmux, sample_m, dG, dG * N, entries - 1 + logN,
                             cpu_query_s)}
    ph = np.array(phases)
    line = {
        "metric": "PSI queries/sec on 1 GB300 (homo_expand + CMUX tree + RLWE blind rotation, bit-exact)",
        "value": value, "unit": "PSI queries/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": statistics.mean(step_ms), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u64", "data": "synthetic",
        "config": {"workload": "the reference PSI test flow at N=2048 (Q=%d, BG=2^%d x%d, Bks_R=2^%d x%d): "
                               "homo_expand of %d packed RLWEs into %d RGSWs, a %d-level CMUX tree over %d "
                               "database RLWEs, an %d-CMUX blind rotation; seeded keys and plaintexts" % (
                                   Q, P.BG_bits, dG, P.Bks_R_bits, L, dG, N, 18 - logN, entries, logN),
                   "l2": "flushed between timed steps (write of a 512 MiB buffer)",
                   "parallelism": "one query per GPU"},
        "e2e": {"value": args.steps / sum(e2e), "unit": "PSI queries/s", "h2d_bytes_per_step": int(packed.nbytes),
                "d2h_bytes_per_step": int(rw * 8), "ms_per_step": 1e3 * statistics.mean(e2e)},
        "phases_ms": {"homo_expand": float(ph[:, 0].mean()), "cmux_tree": float(ph[:, 1].mean()),
                      "blind_rotate": float(ph[:, 2].mean())},
        "roofline": roofline, "cpu_baseline": cpu, "clocks": clk, "gpu_launches": launches,
        "checks": {"result_decodes": bool(decodes(first_out)), "e2e_decodes": bool(e2e_ok),
                   "steps_repeatable": bool(repeat_ok), "setup_s": setup_s},
    }
    if own:
        print(json.dumps(line))
        ctx.close()
    return line


def fheacc_key_bytes(P):
    """Device bytes of the bootstrap + key-switch keys of a parameter set."""
    if P.N == 1024:
        return P.Br * P.digitR * P.n * P.digitG * 4 * P.N * 4 + P.Bks * P.digitKS * P.N * ((P.n + 32) // 32 * 32) * 4
    return P.Br * P.digitR * P.n * P.digitG * 4 * P.N * 16 + P.Bks * P.digitKS * P.N * ((P.n + 32) // 32 * 32) * 8


def config_of(P, batch):
    word = "uint32" if P.N == 1024 else "uint64"
    return {"workload": ("%d independent NAND-gate bootstraps: n=%d, N=%d, Q=%d (%s words), BG=2^%d x%d, "
                         "Br=%d x%d, Bks=%d x%d, q=%d; keys and input bits from fixed seeds") % (
                            batch, P.n, P.N, P.Q, word, P.BG_bits, P.digitG, P.Br, P.digitR, P.Bks, P.digitKS,
                            P.q),
            "batch": batch, "gate": "NAND", "n": P.n, "N": P.N, "Q": P.Q,
            "l2": "flushed between timed steps (write of a 512 MiB buffer); keys (%.1f GB) exceed L2" % (
                (fheacc_key_bytes(P)) / 1e9),
            "parallelism": "one batch per GPU (independent gates, no collective)"}


def extra_blocks(F, D, cache, args, dev_id):
    """The other measured configurations, each with its own CUDA-event
    timing, rooflines and CPU sample, reported inside the default line:
    cfg2, 2048 gates at N = 2048 (64-bit words); mixed, the uneven N = 1024 +
    N = 2048 batch in one CUDA-graph launch; psi, the reference's PSI query at
    N = 2048. Their steps are capped at 3 to keep the whole run within a few
    minutes (the warm-up stays at 3 or more)."""
    import copy
    out = {}
    sub = copy.copy(args)
    sub.steps = min(args.steps, 3)

    def keep(line, keys):
        return {k: line[k] for k in keys if k in line}
    common = ("metric", "value", "unit", "steps", "warmup", "ms_per_step", "dtype", "config", "e2e", "roofline",
              "cpu_baseline", "clocks", "gpu_launches", "checks")
    t0 = time.perf_counter()
    w = measure_batch(F, D, cache, 1, args.wide_batch, sub, dev_id, sub.steps, 2, False)
    out["cfg2"] = keep(w, common + ("roofline_hbm", "plain"))
    out["cfg2"]["wall_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    m = run_mixed(sub, cache)
    out["mixed"] = keep(m, common + ("per_set", "graph_vs_sum_of_alone", "concurrent_branches"))
    out["mixed"]["wall_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    p = run_psi(args, cache)
    out["psi"] = keep(p, common + ("phases_ms",))
    out["psi"]["wall_s"] = time.perf_counter() - t0
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--preset", type=int, default=0)
    ap.add_argument("--plain-sample", type=int, default=48)
    ap.add_argument("--cpu-sample", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extra", action="store_true",
                    help="only the headline configuration (4096 gates, N=1024): skip the cfg2 / mixed / psi blocks")
    ap.add_argument("--wide-batch", type=int, default=2048, help="gates of the N=2048 block (cfg2)")
    ap.add_argument("--serve", action="store_true",
                    help="sweep serving rates (PSI queries through the continuous-batching server) and exit")
    ap.add_argument("--serve-rate", type=float, default=20000.0, help="offered bootstraps/s of the serving sample")
    ap.add_argument("--serve-seconds", type=float, default=8.0)
    ap.add_argument("--psi", action="store_true",
                    help="the reference's PSI query (homo_expand, CMUX tree, RLWE blind rotation) at N=2048 and exit")
    ap.add_argument("--mixed", action="store_true",
                    help="uneven batch of two parameter sets in one CUDA-graph launch (N=1024 + N=2048) and exit")
    ap.add_argument("--mixed-narrow", type=int, default=3000)
    ap.add_argument("--mixed-wide", type=int, default=700)
    ap.add_argument("--mixed-seed", type=int, default=2024)
    ap.add_argument("--profile-case", action="store_true",
                    help="only run the small profiling case (n=64, 912 gates, 2 launches) and exit")
    ap.add_argument("--profile-gates", type=int, default=912, help="gates of the profiling case")
    ap.add_argument("--profile-n", type=int, default=64, help="LWE dimension of the profiling case")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    if args.profile_case:
        return profile_case(args.preset, args.profile_gates, args.profile_n)
    if args.mixed:
        run_mixed(args)
        return 0
    if args.psi:
        run_psi(args)
        return 0

    import torch
    import __graft_entry__
    __graft_entry__.build_product()
    import importlib
    F = importlib.import_module("3rd_gen_fhe_acc_gb300")
    D = Dist(use_cuda=True)
    dev_id = D.local if D.ws > 1 else 0
    torch.cuda.set_device(dev_id)
    cache = KeyCache(F, dev_id)
    line = measure_batch(F, D, cache, args.preset, args.batch, args, dev_id, args.steps, args.plain_sample, True)
    if D.ws == 1 and not args.no_extra:
        line["configs"] = extra_blocks(F, D, cache, args, dev_id)
    if D.rank == 0:
        print(json.dumps(line))
    cache.close()
    D.close()
    return 0


def measure_batch(F, D, cache, preset, B, args, dev_id, n_steps, plain_sample, serve):
    """One batched configuration: K timed steps on device-resident inputs, the
    e2e steps through the host-buffer C ABI, the plain form, the rooflines, a
    CPU sample and (serve) the serving sample; returns the JSON line."""
    import torch
    K = cache.get(preset)
    P, ctx, bt, ks = K["P"], K["ctx"], K["bt"], K["ks"]
    lsk, rsk, x, y, c1, c2, gates = make_inputs(F, P, B, D.rank)
    W = P.n + 1
    stream = torch.cuda.current_stream()
    st = stream.cuda_stream
    d1 = torch.from_numpy(c1.view(np.int64)).cuda()
    d2 = torch.from_numpy(c2.view(np.int64)).cuda()
    dg = torch.from_numpy(gates).cuda()
    dout = torch.zeros_like(d1)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    truth = np.array([F.gate_truth(int(g), a, b) for g, a, b in zip(gates, x, y)], dtype=np.uint8)

    def step_device(profile):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.bootstrap_async(d1.data_ptr(), d2.data_ptr(), dg.data_ptr(), B, dout.data_ptr(),
                            F.FLAG_PROFILE if profile else 0, st)
        e1.record(stream)
        return e0, e1

    # warm-up, device-resident
    for _ in range(args.warmup):
        flush.fill_(1)
        step_device(False)
    torch.cuda.synchronize()
    out0 = dout.cpu().numpy().view(np.uint64).copy()
    dec_ok = int((F.LWE_decrypt(P, lsk, out0) == truth).sum())

    # timed region: K steps, device-resident inputs
    imad = ctx.measure_imad_rate()
    comp = ctx.measure_components() if P.N == 1024 else None
    clocks = ClockSampler(dev_id)
    clocks.start()
    step_ms, br_ms, ks_ms = [], [], []
    D.barrier()
    torch.cuda.synchronize()
    n0 = ctx.kernel_launches()
    for _ in range(n_steps):
        flush.fill_(1)
        e0, e1 = step_device(True)
        torch.cuda.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        b, k = ctx.kernel_times()
        br_ms.append(b)
        ks_ms.append(k)
    launches = ctx.kernel_launches() - n0
    torch.cuda.synchronize()
    D.barrier()
    clk = clocks.stop()
    total_s = D.max(sum(step_ms) / 1e3)
    value = D.ws * B * n_steps / total_s
    same = np.array_equal(dout.cpu().numpy().view(np.uint64), out0)

    # e2e: host buffers through the C ABI (pinned host memory)
    h1 = torch.from_numpy(c1.view(np.int64)).pin_memory()
    h2 = torch.from_numpy(c2.view(np.int64)).pin_memory()
    hg = torch.from_numpy(gates).pin_memory()
    ho = torch.zeros_like(h1).pin_memory()
    n1, n2, ng, no = (t.numpy() for t in (h1, h2, hg, ho))
    e2e_s = []
    for s in range(args.warmup + n_steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = F.lib().fheacc_bootstrap(ctx.handle, n1.ctypes.data_as(F._u64p), n2.ctypes.data_as(F._u64p),
                                     ng.ctypes.data_as(F._i32p), B, no.ctypes.data_as(F._u64p), 0)
        dt = time.perf_counter() - t0
        ctx.check(r)
        if s >= args.warmup:
            e2e_s.append(dt)
    D.barrier()
    e2e_total = D.max(sum(e2e_s))
    e2e_value = D.ws * B * n_steps / e2e_total
    e2e_same = np.array_equal(no.view(np.uint64), out0)

    # plain form: one launch sequence per gate
    Pn = min(plain_sample, B)
    ctx.bootstrap_plain_async(d1.data_ptr(), d2.data_ptr(), dg.data_ptr(), 4, dout.data_ptr(), 0, st)
    torch.cuda.synchronize()
    lat = []
    for i in range(Pn):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        off = i * W
        ctx.bootstrap_plain_async(d1.data_ptr() + 8 * off, d2.data_ptr() + 8 * off, dg.data_ptr() + 4 * i, 1,
                                  dout.data_ptr() + 8 * off, 0, st)
        e1.record(stream)
        torch.cuda.synchronize()
        lat.append(e0.elapsed_time(e1))
    plain_value = Pn / (sum(lat) / 1e3)
    plain_ok = np.array_equal(dout.cpu().numpy().view(np.uint64)[:Pn], out0[:Pn])

    # roofline of the dominant kernel (blind rotation)
    steps = steps_of(c1, c2, gates, P)
    total_steps = int(steps.sum())
    N, dG = P.N, P.digitG
    logN = N.bit_length() - 1
    # 2 inverse + 2*digitG forward NTTs, the MAC products, and the N^-1 scaling
    # of the two inverse NTTs: 69,632 per step for this parameter set
    modmul_per_step = (2 + 2 * dG) * (N // 2) * logN + 2 * (2 * dG) * N + 2 * N
    br_s = statistics.mean(br_ms) / 1e3
    achieved_modmul = total_steps * modmul_per_step / br_s
    # IMAD issue slots per Shoup modular multiply: 32-bit words 4 (mul.hi counts
    # 2); 64-bit words 16 (the 128-bit quotient estimate takes three wide and one
    # high 32-bit product, each 2 slots, and the two low 64-bit products 4 each)
    slots = 4.0 if N == 1024 else 16.0
    peak_modmul = imad / slots
    word = 4 if N == 1024 else 8
    rgsw_bytes = 2 * dG * 2 * N * word
    btkey_bytes = P.Br * P.digitR * P.n * rgsw_bytes
    traffic = None
    if os.path.exists(TRAFFIC_FILE):
        with open(TRAFFIC_FILE) as f:
            tj = json.load(f)
        if B == 4096 and preset == 0:
            traffic = tj.get("br32_pipe", {}).get("bytes_per_launch_4096")
        elif B == 2048 and preset == 1:
            traffic = tj.get("br64", {}).get("bytes_per_launch_2048")
    hbm_peak = None
    peaks_src = "fallback 6800 GB/s"
    if os.path.exists(PEAKS_FILE):
        with open(PEAKS_FILE) as f:
            hbm_peak = json.load(f).get("hbm_gbs")
            peaks_src = "measured (MEASURED_PEAKS.json hbm_gbs)"
    hbm_peak = hbm_peak or 6800.0
    key_stream_gbs = total_steps * rgsw_bytes / br_s / 1e9
    l2_peak_gbs = ctx.measure_l2_read_rate() / 1e9
    # plain form: one gate per launch sequence streams its own RGSW per step
    # and its key-switch rows; the mean gate of the sample
    ks_rows = P.N * P.digitKS
    plain_bytes = float(steps[:Pn].mean()) * rgsw_bytes + ks_rows * (P.n + 1) * word
    plain_gbs = plain_bytes / (statistics.mean(lat) / 1e3) / 1e9
    roofline = {
        "bound": "int", "achieved": achieved_modmul / 1e9, "peak": peak_modmul / 1e9, "unit": "G modmul/s",
        "frac": achieved_modmul / peak_modmul, "traffic": traffic,
        "kernel": "br32_pipe_kernel" if N == 1024 else "br64_kernel", "kernel_ms": statistics.mean(br_ms),
        "work": "%d RLWE x RGSW steps x %d modular multiplies (NTT butterflies, MAC products, N^-1 scaling)" % (
            total_steps, modmul_per_step),
        "peak_source": "IMAD rate measured in this run (%.1f T lane-op/s) / %d IMAD issue slots per %d-bit Shoup "
                       "modular multiply" % (imad / 1e12, slots, 32 if N == 1024 else 64),
    }
    if comp:
        # SM time of one step's pieces run alone vs the pipeline's SM time per step
        sms = torch.cuda.get_device_properties(dev_id).multi_processor_count
        # the last digit's NTT comes from the accumulator when Q < BG^digitG
        derive = (P.Q >> (P.BG_bits * dG)) == 0
        step_sum = 2 * (dG - (1 if derive else 0)) * comp["ntt_digit"] + 2 * comp["intt"] + comp["mac"]
        step_pipe = br_s * 1e9 * sms / total_steps
        roofline["components"] = {
            "unit": "SM ns per unit, each piece run alone at the kernel's occupancy (fheacc_measure_components)",
            "ntt_fwd_ns": comp["ntt_fwd"], "ntt_digit_ns": comp["ntt_digit"], "intt_ns": comp["intt"],
            "mac_step_ns": comp["mac"], "step_sum_ns": step_sum, "step_pipeline_ns": step_pipe,
            "overlap_frac": step_sum / step_pipe}
    roofline_hbm = {
        "bound": "hbm", "achieved": btkey_bytes / br_s / 1e9, "peak": hbm_peak, "unit": "GB/s",
        "frac": btkey_bytes / br_s / 1e9 / hbm_peak, "traffic": traffic,
        "algorithmic_bytes": btkey_bytes, "peak_source": peaks_src,
        "plain": {"achieved": plain_gbs, "frac": plain_gbs / hbm_peak, "algorithmic_bytes_per_gate": plain_bytes,
                  "note": "one gate per launch sequence: its RGSW per step and its key-switch rows, over the "
                          "plain latency"},
        "target_60pct_met": False,
        "note": "batched: algorithmic bytes = the bootstrap key read once per launch; the batch shares every key "
                "tile, so the launch is bound by the integer multiply pipe and its HBM fraction is small by "
                "construction. Plain: one gate's steps are a serial chain of RLWE x RGSW products on one SM, "
                "latency-bound. Neither form reaches 60% of HBM.",
    }
    roofline_l2 = {
        "bound": "l2", "achieved": key_stream_gbs, "peak": l2_peak_gbs, "unit": "GB/s",
        "frac": key_stream_gbs / l2_peak_gbs,
        "algorithmic_bytes": total_steps * rgsw_bytes,
        "peak_source": "fheacc_measure_l2_read_rate in this run: every SM streaming a buffer of a third of L2 "
                       "with 16-byte L2-only loads",
        "note": "key streaming: the RGSW bytes all steps of all gates consume (each gate reads its residue's "
                "RGSW every step), served from L2",
    }

    cpu = None
    if D.rank == 0 and D.ws == 1 and not args.no_cpu:
        import __graft_entry__ as ge
        ge._build_oracle()
        from oracle_lib import Oracle
        ora = Oracle.from_params(P)
        cores = cpu_cores()
        nsample = args.cpu_sample or (8 if P.N == 1024 else 2) * cores
        t0 = time.perf_counter()
        co, failed = ora.eval_bootstrap_batch(c1[:nsample], c2[:nsample], gates[:nsample], bt, ks, threads=cores)
        dt = time.perf_counter() - t0
        cpu = {"value": nsample / dt, "unit": "bootstraps/s", "cores": cores, "kind": "port",
               "sample": "first %d gates of the batch, oracle eval_bootstrap (C restatement of "
                         "RLWE.cpp:726-786) on %d threads, %.1f s" % (nsample, cores, dt),
               "bitexact_vs_gpu": "%d/%d" % (int((co == out0[:nsample]).all(axis=1).sum()), nsample)}

    serving = None
    if serve and D.ws == 1 and args.serve_seconds > 0 and P.N == 1024:   # the server runs the 32-bit sets
        serving = run_serving(F, ctx, P, lsk, args.serve_rate, args.serve_seconds)
    if serve and args.serve and P.N == 1024:
        sweep = [run_serving(F, ctx, P, lsk, r, 10.0) for r in (1e3, 5e3, 1e4, 2e4, 3e4, 4e4, 6e4, 1e5)]
        print(json.dumps({"serving_sweep": sweep}))

    line = {
        "metric": METRIC, "value": value, "unit": "bootstraps/s", "n_gpus": D.ws, "steps": n_steps,
        "warmup": args.warmup, "ms_per_step": statistics.mean(step_ms), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32" if P.N == 1024 else "u64", "data": "synthetic",
        "config": config_of(P, B),
        "e2e": {"value": e2e_value, "unit": "bootstraps/s",
                "h2d_bytes_per_step": int(2 * B * W * 8 + B * 4), "d2h_bytes_per_step": int(B * W * 8),
                "ms_per_step": 1e3 * statistics.mean(e2e_s)},
        "roofline": roofline, "roofline_hbm": roofline_hbm, "roofline_l2": roofline_l2,
        "cpu_baseline": cpu, "clocks": clk,
        "gpu_launches": launches * D.ws,
        "plain": {"value": plain_value, "unit": "bootstraps/s", "gates": Pn,
                  "latency_ms_p50": statistics.median(lat), "latency_ms_p99": float(np.percentile(lat, 99)),
                  "batched_over_plain": value / plain_value / D.ws},
        "batch_latency_ms_p50": statistics.median(step_ms), "batch_latency_ms_p99": float(np.percentile(step_ms, 99)),
        "serving": serving,
        "checks": {"decrypt_ok": "%d/%d" % (dec_ok, B), "steps_repeatable": bool(same), "e2e_equal": bool(e2e_same),
                   "plain_equal": bool(plain_ok), "kernel_ms": {"blind_rotate": statistics.mean(br_ms),
                                                                "keyswitch": statistics.mean(ks_ms)}},
    }
    return line


if __name__ == "__main__":
    sys.exit(main())
