"""Benchmark: random-forest build on one GB300 (and N independent replicas).

Workload (the headline configuration): RF multiclass with bootstrap,
1,000,000 rows x 128 FP32 features (N(0,1), 16 of them integers 0..15 stored as
float), 10 classes, 128 trees, entropy, 11 features tried per node, max depth
20, min leaf 2 (min node size 5, the reference default).  Seeded synthetic data.

A step is one complete forest fit.  ``value`` is forest-build throughput in
nodes/s (internal + leaf nodes created per second of device time) with the
samples already resident in HBM; ``e2e`` is the same metric through the C ABI
with pinned host buffers (the samples' upload and the model's download inside
the timed region).  ``--impl reference`` times the reference path's CPU
restatement on the host cores (the reference itself has no CPU path).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import gc
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

WORKLOAD = dict(name="rf_multiclass_1Mx128_c10_128trees", rows=1_000_000, features=128,
                classes=10, n_int=16, trees=128, K=11, max_depth=20, min_node_size=5,
                min_leaf=2, seed=0)
SMALL = dict(WORKLOAD, name="rf_multiclass_200kx64_c10_32trees", rows=200_000, features=64,
             trees=32)


def fit_kwargs(w):
    return dict(algo=0, task=0, n_trees=w["trees"], K=w["K"], max_depth=w["max_depth"],
                min_node_size=w["min_node_size"], min_leaf=w["min_leaf"],
                n_classes=w["classes"], seed=w["seed"])


def make_data(w):
    from datamininglibs_gb300 import synth
    return synth.rf_multiclass(w["rows"], w["features"], n_classes=w["classes"],
                               n_int=w["n_int"], seed=w["seed"])


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def host_link_rate(torch, mib=256):
    """Copy rate between pinned host memory and the device (GB/s, CUDA events on
    one 256 MiB copy each way).  The end-to-end fit and the serving leg move
    their samples, models and requests over this link, and its rate has varied
    between boxes and over time (other jobs share the host), so it is reported
    beside the numbers that depend on it."""
    n = mib << 18
    d = torch.empty(n, dtype=torch.float32, device="cuda")
    h = torch.empty(n, dtype=torch.float32, pin_memory=True)
    h.fill_(1.0)
    out = {}
    for key, dst, src in (("h2d", d, h), ("d2h", h, d)):
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        dst.copy_(src, non_blocking=True)
        b.record()
        torch.cuda.synchronize()
        out[key] = round(n * 4 / (a.elapsed_time(b) * 1e6), 1)
    return out


def traffic_from_profile(kernel):
    """DRAM bytes per tried entry of a search kernel, measured by ncu on the
    200k x 64 case (profiles/search_kernels_rf_multiclass.md, lines
    `dram_bytes_per_entry_try <kernel>: <bytes>`); scaled to a launch by the
    launch's tried entries."""
    path = os.path.join(ROOT, "profiles", "search_kernels_rf_multiclass.md")
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_entry_try " + kernel + ":"):
                return float(line.split(":")[-1])
    except OSError:
        pass
    return None


def cpu_baseline(w, X, y, threads, trees, with_model=False):
    """The oracle (CPU restatement of the reference path) on all host threads,
    on the full-size data: ``trees`` of the workload's trees (one per thread
    when trees >= threads, otherwise the nodes of a level spread over threads)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    kw = fit_kwargs(w)
    kw["n_trees"] = trees
    t0 = time.perf_counter()
    m = oracle.fit(X, y, threads=threads, **kw)
    dt = time.perf_counter() - t0
    cb = {"value": m.nodes.shape[0] / dt, "unit": "nodes/s", "cores": threads,
          "kind": "port", "sample": "%d of the %d trees on the full %dx%d data (%.1f s)" % (
              trees, w["trees"], w["rows"], w["features"], dt)}
    return (cb, m) if with_model else cb


def oracle_rate(fn, what, threads):
    """nodes/s of one oracle fit (all host threads) on a bounded sample."""
    t0 = time.perf_counter()
    nodes = fn()
    dt = time.perf_counter() - t0
    return {"value": nodes / dt, "unit": "nodes/s", "cores": threads, "kind": "port",
            "sample": "%s (%.1f s)" % (what, dt)}


def other_cpu_baselines(threads):
    """The oracle on all host threads for the other workloads, each a bounded
    sample of the workload on its full data (nodes/s)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from datamininglibs_gb300 import synth
    out = {}
    X1, y1 = synth.ert_binary()

    def c1():
        n = 0
        for _ in range(5):
            n += oracle.fit(X1, y1, algo=1, n_trees=64, K=7, max_depth=12, min_node_size=10,
                            n_classes=2, seed=0, threads=threads).nodes.shape[0]
        return n
    out["ert_binary_4601x57_64trees"] = oracle_rate(c1, "5 fits of the whole 64-tree forest",
                                                    threads)
    probs = synth.uneven_problems(256, seed=0)

    def c4():
        return sum(oracle.fit(X, y, algo=1, n_trees=2, K=0, max_depth=16, min_node_size=5,
                              n_classes=c, seed=i, threads=threads).nodes.shape[0]
                   for i, (X, y, c) in enumerate(probs))
    out["uneven_256_ert_forests"] = oracle_rate(
        c4, "trees 0-1 of each of the 256 forests (16 trees each in the workload)", threads)
    del probs
    X3, y3 = synth.rf_regression()
    X3 = np.ascontiguousarray(X3[:, :1_000_000])
    y3 = np.ascontiguousarray(y3[:1_000_000])

    def c3():
        return oracle.fit(X3, y3, algo=0, task=1, n_trees=1, K=21, max_depth=24, min_node_size=5,
                          min_leaf=5, seed=0, threads=threads).nodes.shape[0]
    out["rf_regression_4Mx64_64trees"] = oracle_rate(
        c3, "tree 0 of the 64 on the first 1,000,000 of the 4,000,000 rows (a tree on all "
            "rows takes about 110 s on 16 Grace cores)", threads)
    return out


def parity_of_timed_forest(w, nodes, probs, gains, m):
    """Trees 0.. of the timed forest against the oracle's fit of the same
    workload's first trees (its cpu_baseline sample), tree by tree in
    breadth-first form: structure, thresholds and leaf class counts bit for bit;
    the engine's FP32 split gains bit for bit against the oracle's FP32 gains and
    within 1e-6 relative + 1e-7 of its FP64 gains."""
    from datamininglibs_gb300 import model
    C = w["classes"]
    exact = gains_exact = within = True
    worst = 0.0
    for t in range(m.n_trees):
        en, ep, eg = model.tree_arrays(nodes, probs, C, t, gains)
        on, op, og32 = model.tree_arrays(m.nodes, m.probs, C, t, m.gains32)
        og64 = model.tree_arrays(m.nodes, m.probs, C, t, m.gains64)[2]
        same = en.shape == on.shape and np.array_equal(en, on) and np.array_equal(ep, op)
        exact = exact and same
        if same:
            sp = on[:, 1] > 0
            gains_exact = gains_exact and np.array_equal(eg[sp].view(np.uint32),
                                                         og32[sp].view(np.uint32))
            err = np.abs(eg[sp].astype(np.float64) - og64[sp])
            within = within and bool(np.all(err <= 1e-6 * np.abs(og64[sp]) + 1e-7))
            big = np.abs(og64[sp]) > 1e-6
            if big.any():
                worst = max(worst, float((err[big] / np.abs(og64[sp][big])).max()))
    return {"config": w["name"], "trees": m.n_trees, "bit_exact": bool(exact),
            "gains_fp32_bit_exact": bool(gains_exact),
            "gains_within_1e-6_rel_1e-7_abs_of_fp64": bool(within),
            "gains_max_rel_err_vs_fp64": worst,
            "compared": "trees 0..%d of the last timed %d-tree forest vs the oracle's "
                        "cpu_baseline fit" % (m.n_trees - 1, w["trees"])}


def run_reference(args, w):
    """The reference path's CPU restatement timed on the host cores.  A timed
    step builds as many of the workload's trees as there are host threads, one
    tree per thread (the way the CPU is used best); a warm-up step builds one."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    X, y = make_data(w)
    threads = os.cpu_count() or 1
    trees = min(threads, w["trees"])
    for _ in range(args.warmup):
        cpu_baseline(w, X, y, threads, 1)
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vals.append(cpu_baseline(w, X, y, threads, trees))
    total = time.perf_counter() - t0
    value = float(np.mean([v["value"] for v in vals]))
    cb = dict(vals[-1])
    cb["value"] = value
    line = {"impl": "reference", "metric": "rf_build_nodes_per_s", "value": value,
            "unit": "nodes/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * total / max(1, args.steps), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
            "config": {"workload": w["name"],
                       "sample": "%d of the %d trees per step, one per host thread" % (
                           trees, w["trees"])},
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": "nodes/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def batched_leg(dml, torch, stream):
    """256 uneven ERT problems (rows log-uniform 200..50,000, features 8..256,
    2..8 classes, 16 trees each, depth 16, min node size 5) fitted together,
    one at a time, and with the plain chunked launch structure."""
    from datamininglibs_gb300 import synth
    probs = synth.uneven_problems(256, seed=0)
    specs = [dict(X=torch.from_numpy(X).cuda(), y=torch.from_numpy(y).cuda(), algo=1,
                  n_trees=16, K=0, max_depth=16, min_node_size=5, n_classes=c, seed=i)
             for i, (X, y, c) in enumerate(probs)]
    for _ in range(2):
        for f in dml.fit_batched(specs, stream=stream):
            f.free()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    reps = 3
    for _ in range(reps):
        fs = dml.fit_batched(specs, stream=stream)
        nodes = sum(f.info().n_nodes for f in fs)
        keep = fs[:32]
        for f in fs[32:]:
            f.free()
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / reps

    def one_by_one(fn):
        torch.cuda.synchronize()
        t = time.perf_counter()
        for sp in specs:
            sp = dict(sp)
            X, y = sp.pop("X"), sp.pop("y")
            fn(X, y, stream=stream, **sp).free()
        torch.cuda.synchronize()
        return time.perf_counter() - t
    t_single = one_by_one(dml.fit)
    t_plain = one_by_one(dml.fit_plain)
    return {"workload": "256 uneven ERT forests x 16 trees", "nodes": nodes,
            "nodes_per_s": nodes / dt, "ms": dt * 1e3,
            "one_at_a_time_nodes_per_s": nodes / t_single,
            "plain_path_nodes_per_s": nodes / t_plain,
            "speedup_vs_plain": t_plain / dt}, keep, probs[:32]


def serve_leg(dml, torch, stream, c2_forest, c4_forests, c4_probs):
    """Resident forests (the ERT binary, RF multiclass and RF regression
    workloads plus 32 of the uneven forests), Poisson arrivals at 100k req/s
    offered, request rows log-uniform in [1, 65536], forest chosen uniformly.
    Also returns the device time of the ERT binary and RF regression fits
    (their samples resident, after one untimed fit)."""
    from datamininglibs_gb300 import synth

    def timed_fit(X, y, **kw):  # device-resident samples; a second, timed fit
        Xd, yd = torch.from_numpy(X).cuda(), torch.from_numpy(y).cuda()
        dml.fit(Xd, yd, stream=stream, **kw).free()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        f = dml.fit(Xd, yd, stream=stream, **kw)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        return f, {"ms": ms, "nodes": f.info().n_nodes,
                   "nodes_per_s": f.info().n_nodes / (ms / 1000.0)}
    X1, y1 = synth.ert_binary()
    f1, fit1 = timed_fit(X1, y1, algo=1, n_trees=64, K=7, max_depth=12, min_node_size=10,
                         n_classes=2, seed=0)
    X3, y3 = synth.rf_regression()
    f3, fit3 = timed_fit(X3, y3, algo=0, task=1, n_trees=64, K=21, max_depth=24,
                         min_node_size=5, min_leaf=5, seed=0)
    del X3, y3
    configs = {"ert_binary_4601x57_64trees_fit": fit1, "rf_regression_4Mx64_64trees_fit": fit3}
    forests = [(f1, "ert_binary"), (c2_forest, "rf_multiclass"), (f3, "rf_regression")]
    forests += [(f, "normal") for f in c4_forests]
    rng = np.random.default_rng(5)

    def pinned(n):  # request rows and results live in pinned host memory
        return torch.empty(n, dtype=torch.float32, pin_memory=True).numpy()
    pools = {}
    for k in ("ert_binary", "rf_regression", "normal"):
        pools[k] = pinned(65536 * 256)
        pools[k][:] = synth.request_rows(rng, 65536, 256, k).reshape(-1)
    pools["rf_multiclass"] = pools["normal"]
    srv = dml.Server(hbm_budget_bytes=4 << 30, max_batch_rows=1 << 16, n_streams=4,
                     max_wait_us=20, small_rows=4096)
    fids = [srv.add_forest(f) for f, _ in forests]
    infos = [f.info() for f, _ in forests]
    ring = pinned(1 << 26)
    M = 6000
    rate = 100_000.0

    def burst(seed, M=M):
        """M requests with Poisson arrivals at `rate`; per-request latency
        (submit to completion, measured by the server) and the burst's rows/s
        from the first submit to the last completion.  Python's garbage
        collector is held off while the requests are submitted, so that a
        collection does not delay the arrivals."""
        r = np.random.default_rng(seed)
        arrivals = np.cumsum(r.exponential(1.0 / rate, M))
        sizes = np.exp(r.uniform(0.0, np.log(65536.0), M)).astype(np.int64)
        which = r.integers(0, len(forests), M)
        reqs = []
        for i in range(M):
            fi = int(which[i])
            F = infos[fi].n_features
            n = int(sizes[i])
            X = pools[forests[fi][1]][: F * n].reshape(F, n)
            width = infos[fi].n_classes
            off = (i * 997 * 64) % (ring.size - n * width)
            reqs.append((fi, X, ring[off: off + n * width].reshape(n, width), n))
        gc.collect()
        gc.disable()
        try:
            t0 = time.perf_counter()
            ids, sub_t = [], []
            for i, (fi, X, out, n) in enumerate(reqs):
                while time.perf_counter() - t0 < arrivals[i]:
                    pass
                sub_t.append(time.perf_counter() - t0)
                ids.append(srv.submit(fids[fi], X, out))
            t_submit = time.perf_counter() - t0
            lat = np.array([srv.wait(q) for q in ids])
        finally:
            gc.enable()
        done = np.array(sub_t) + lat / 1000.0
        rows = np.array([q[3] for q in reqs])
        small = rows <= 4096
        return reqs, {
            "requests": M, "offered_req_per_s": M / t_submit,
            "offered_rows_per_s": float(rows.sum()) / t_submit,
            "rows_per_s": float(rows.sum()) / float(done.max() - sub_t[0]),
            "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "le4k_requests": int(small.sum()),
            "p50_ms_le4k": float(np.percentile(lat[small], 50)),
            "p99_ms_le4k": float(np.percentile(lat[small], 99))}
    # an untimed warm-up burst of the timed bursts' size: the server's first
    # batches load its kernels and touch its streams and buffers for the first
    # time (the link probe's pinned buffer is allocated before it)
    host_link_rate(torch)
    burst(4)
    bursts = []
    for rep in range(3):
        link = host_link_rate(torch)
        reqs, b = burst(5 + rep)
        b["host_link_GBps_before"] = link
        bursts.append(b)
    st = srv.stats()
    srv.close()
    # the plain path: each request alone through the reference's predict
    # structure (dml_predict_plain), one after another, on a sample of the stream
    torch.cuda.synchronize()
    tp = time.perf_counter()
    rows = 0
    for fi, X, out, n in reqs[:600]:
        forests[fi][0].predict_plain(X, out=out)
        rows += n
    plain_rows_per_s = rows / (time.perf_counter() - tp)
    f1.free()
    f3.free()
    served = float(np.median([b["rows_per_s"] for b in bursts]))
    return {"bursts": bursts, "requests_per_burst": M,
            "offered": "Poisson arrivals at %.0f req/s, rows log-uniform in [1, 65536] "
                       "(about %.0f M rows/s offered, above what the server completes, so "
                       "the large-request queue grows during a burst)" % (
                           rate, np.mean([b["offered_rows_per_s"] for b in bursts]) / 1e6),
            "rows_per_s": served, "small_rows": 4096,
            "p50_ms_le4k": float(np.median([b["p50_ms_le4k"] for b in bursts])),
            "p99_ms_le4k_max": float(max(b["p99_ms_le4k"] for b in bursts)),
            "server": "one server, an untimed warm-up burst, then three bursts of %d "
                      "requests, idle between bursts" % M,
            "plain": "dml_predict_plain on the first 600 requests of the last burst",
            "launches": st.launches, "plain_rows_per_s": plain_rows_per_s,
            "speedup_vs_plain": served / plain_rows_per_s}, configs


def run_ours(args, w):
    import torch

    import datamininglibs_gb300 as dml
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dml.lib()
    X, y = make_data(w)
    Xd = torch.from_numpy(X).cuda()
    yd = torch.from_numpy(y).cuda()
    kw = fit_kwargs(w)
    stream = torch.cuda.current_stream()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    # scheduling picked by the autotuner on a 32-tree sample (untimed)
    tuning = None if args.no_tune else dml.autotune(Xd, yd, sample_trees=32, stream=stream, **kw)
    for _ in range(args.warmup):
        dml.fit(Xd, yd, stream=stream, **kw).free()
    barrier()
    clk = ClockSampler(local)
    clk.start()
    time.sleep(0.3)
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    nodes = entries = entry_tries = launches = 0
    search_ms = loop_ms = 0.0
    nq = dml.ensembles.NUM_QUEUES
    q_ms, q_ent, q_tries, q_launch = [0.0] * nq, [0] * nq, [0] * nq, [0] * nq
    e0.record(stream)
    for _ in range(args.steps):
        f = dml.fit(Xd, yd, stream=stream, **kw)
        st = dml.ensembles.last_fit_stats()
        nodes += st.nodes
        entries += st.entries
        entry_tries += st.entry_tries
        launches += st.launches
        search_ms += st.search_ms
        loop_ms += st.level_loop_ms
        for q in range(nq):
            q_ms[q] += st.queue_ms[q]
            q_ent[q] += st.queue_entries[q]
            q_tries[q] += st.queue_entry_tries[q]
            q_launch[q] += st.queue_launches[q]
        last_forest = f
        if _ != args.steps - 1:
            f.free()
    e1.record(stream)
    barrier()
    clocks = clk.stop()
    dev_ms = e0.elapsed_time(e1)
    t_all = torch.tensor([dev_ms, float(nodes)], dtype=torch.float64, device="cuda")
    if dist is not None:
        mx = t_all.clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        tot = t_all.clone()
        dist.all_reduce(tot, op=dist.ReduceOp.SUM)
        dev_ms, nodes_all = mx[0].item(), tot[1].item()
    else:
        nodes_all = float(nodes)
    value = nodes_all / (dev_ms / 1000.0)

    # predict throughput with the last forest (rows resident, > L2)
    pe0 = torch.cuda.Event(enable_timing=True)
    pe1 = torch.cuda.Event(enable_timing=True)
    out = torch.empty((w["rows"], w["classes"]), dtype=torch.float32, device="cuda")
    last_forest.predict(Xd, out=out, stream=stream)
    torch.cuda.synchronize()
    pe0.record(stream)
    for _ in range(3):
        last_forest.predict(Xd, out=out, stream=stream)
    pe1.record(stream)
    torch.cuda.synchronize()
    predict_rows_per_s = 3 * w["rows"] / (pe0.elapsed_time(pe1) / 1000.0)
    finfo = last_forest.info()
    predict_roofline = None
    if rank == 0:
        from datamininglibs_gb300 import model
        pn, pp = last_forest.export()
        path = model.mean_path_nodes(pn, pp, w["trees"], w["classes"])
        del pn, pp
        io_b = 4 * w["features"] + 4 * w["classes"]
        # bulk prediction walks the compact 8-byte nodes (16-byte with DML_PREDICT_NODE16)
        node_size = 16 if os.environ.get("DML_PREDICT_NODE16", "0") not in ("", "0") else 8
        node_b = node_size * w["trees"] * path
        peak, peak_kind = measured_peak()
        predict_roofline = {
            "bound": "hbm", "unit": "GB/s", "peak": peak, "peak_kind": peak_kind,
            "rows_per_s": predict_rows_per_s,
            "io_bytes_per_row": io_b,
            "mean_nodes_per_tree": path,
            "node_bytes_per_row": node_b,
            "achieved_io": predict_rows_per_s * io_b / 1e9,
            "frac_io": predict_rows_per_s * io_b / 1e9 / peak,
            "achieved_with_nodes": predict_rows_per_s * (io_b + node_b) / 1e9,
            "frac_with_nodes": predict_rows_per_s * (io_b + node_b) / 1e9 / peak,
            "node_bytes": node_size,
            "note": "io = 4F + 4C bytes per row (row read once, votes written once); nodes = "
                    "trees x mean nodes per walk x %d-byte predict nodes (loads, many from L2: "
                    "the forest's predict nodes are %.0f MB)" % (node_size,
                                                                 finfo.n_nodes * node_size / 1e6)}

    # e2e: the C ABI with pinned host buffers, upload and model download timed.
    # The model is read into pinned buffers allocated once, as a caller that
    # fits repeatedly would keep them; every fit of this seeded workload gives
    # the forest of the timed fits, so they take its sizes.
    Xh = torch.from_numpy(X).pin_memory()
    yh = torch.from_numpy(y).pin_memory()
    nbuf = torch.empty((finfo.n_nodes, 5), dtype=torch.int32, pin_memory=True).numpy()
    pbuf = torch.empty(finfo.n_probs, dtype=torch.float32, pin_memory=True).numpy()
    e2e_steps = max(1, min(args.steps, 3))
    link_before = host_link_rate(torch)
    barrier()
    t0 = time.perf_counter()
    e2e_nodes = 0
    d2h = 0
    for _ in range(e2e_steps):
        f = dml.fit(Xh, yh, stream=stream, **kw)
        nd, pr = f.export(nbuf, pbuf)
        e2e_nodes += nd.shape[0]
        d2h += nd.nbytes + pr.nbytes
        f.free()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    link_after = host_link_rate(torch)
    h2d = X.nbytes + y.nbytes

    extras = {}
    if world == 1 and not args.no_extras:
        # the reference-structured plain path on the same workload
        torch.cuda.synchronize()
        tp = time.perf_counter()
        fp = dml.fit_plain(Xd, yd, stream=stream, **kw)
        torch.cuda.synchronize()
        extras["plain_path"] = {"nodes_per_s": fp.info().n_nodes / (time.perf_counter() - tp)}
        fp.free()
        extras["batched_uneven"], c4f, c4p = batched_leg(dml, torch, stream)
        extras["serve"], extras["other_configs"] = serve_leg(dml, torch, stream, last_forest,
                                                             c4f, c4p)
        for f in c4f:
            f.free()
    keep_model = world == 1 and not args.no_cpu
    if keep_model:
        timed_nodes, timed_probs = last_forest.export()
        timed_gains = last_forest.gains()
    last_forest.free()
    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return
    peak, peak_kind = measured_peak()
    # the dominant kernel: the node class with the most device time; its
    # algorithmic bytes (4 per tried entry, 20 per searched entry) over its
    # CUDA-event time on the fit stream
    names = dml.ensembles.QUEUE_KERNELS
    dom = max(range(nq), key=lambda q: q_ms[q])
    alg_q = [4.0 * q_tries[q] + 20.0 * q_ent[q] for q in range(nq)]
    achieved = alg_q[dom] / (q_ms[dom] / 1000.0) / 1e9 if q_ms[dom] > 0 else None
    tpu = traffic_from_profile(names[dom])
    queues = {names[q]: {"ms_per_fit": q_ms[q] / args.steps,
                         "share": q_ms[q] / search_ms if search_ms > 0 else None,
                         "launches_per_fit": q_launch[q] / args.steps,
                         "algorithmic_GBps": alg_q[q] / (q_ms[q] / 1000.0) / 1e9}
              for q in range(nq) if q_ms[q] > 0}
    line = {
        "metric": "rf_build_nodes_per_s", "value": value, "unit": "nodes/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
        "config": {"workload": w["name"], "rows": w["rows"], "features": w["features"],
                   "classes": w["classes"], "trees": w["trees"], "features_per_node": w["K"],
                   "max_depth": w["max_depth"], "min_leaf": w["min_leaf"],
                   "min_node_size": w["min_node_size"],
                   "l2": "inputs larger than L2 (%.0f MB of samples)" % (X.nbytes / 1e6),
                   "parallelism": "replicas" if world > 1 else "single",
                   "tuning": tuning},
        "trees_per_s": world * args.steps * w["trees"] / (dev_ms / 1000.0),
        "nodes_per_fit": nodes / args.steps,
        "predict_rows_per_s": predict_rows_per_s,
        "predict_roofline": predict_roofline,
        "forest": {"nodes": finfo.n_nodes, "max_depth": finfo.max_depth},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None,
                     "traffic": (tpu * q_tries[dom] / max(1, q_launch[dom])) if tpu else None,
                     "kernel": names[dom],
                     "algorithmic_bytes_per_launch": alg_q[dom] / max(1, q_launch[dom]),
                     "launches": q_launch[dom],
                     "peak_kind": peak_kind,
                     "search_ms_per_fit": search_ms / args.steps,
                     "level_loop_ms_per_fit": loop_ms / args.steps,
                     "search_algorithmic_GBps": (4.0 * entry_tries + 20.0 * entries)
                     / (search_ms / 1000.0) / 1e9 if search_ms > 0 else None},
        "search_kernels": queues,
        "e2e": {"value": e2e_nodes / e2e_s, "unit": "nodes/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h // e2e_steps},
        "host_link_GBps": {"before_e2e": link_before, "after_e2e": link_after,
                           "note": "pinned host <-> device copy rate, 256 MiB each way"},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    line.update(extras)
    if keep_model:
        th = os.cpu_count() or 1
        line["cpu_baseline"], m = cpu_baseline(w, X, y, th, min(th, w["trees"]), with_model=True)
        line["parity"] = parity_of_timed_forest(w, timed_nodes, timed_probs, timed_gains, m)
        del timed_nodes, timed_probs, timed_gains, m
        if "other_configs" in line:
            line["other_configs"]["cpu_baselines"] = other_cpu_baselines(th)
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def run_predict_file(args, w):
    """--save-forest: fit the workload's forest once and save it.  --predict-from:
    load a saved forest and predict the workload's rows (resident on the
    device) 3 times after one warm-up; prints rows/s.  The predict process then
    holds only the forest, the rows and the votes (a few GB), the size an ncu
    capture of the predict kernel wants."""
    import torch

    import datamininglibs_gb300 as dml
    dml.lib()
    X, y = make_data(w)
    if args.save_forest:
        f = dml.fit(X, y, **fit_kwargs(w))
        f.save(args.save_forest)
        print(json.dumps({"saved": args.save_forest, "nodes": f.info().n_nodes}), flush=True)
        return
    f = dml.Forest.load(args.predict_from)
    Xd = torch.from_numpy(X).cuda()
    out = torch.empty((w["rows"], w["classes"]), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    f.predict(Xd, out=out, stream=stream)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(3):
        f.predict(Xd, out=out, stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    print(json.dumps({"predict_rows_per_s": 3 * w["rows"] / (e0.elapsed_time(e1) / 1000.0),
                      "nodes": f.info().n_nodes}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--small", action="store_true", help="a reduced workload for quick checks")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-tune", action="store_true",
                    help="skip the autotuner (default scheduling; for ncu launch indices)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the plain-path, batched-forest and serving legs")
    ap.add_argument("--save-forest", default=None,
                    help="fit the workload's forest once, save it to this file, exit")
    ap.add_argument("--predict-from", default=None,
                    help="load a saved forest and time predict on the workload's rows, exit")
    args = ap.parse_args()
    w = SMALL if args.small else WORKLOAD
    if args.save_forest or args.predict_from:
        run_predict_file(args, w)
    elif args.impl == "reference":
        run_reference(args, w)
    else:
        run_ours(args, w)


if __name__ == "__main__":
    main()
