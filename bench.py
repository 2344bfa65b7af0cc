"""Benchmark of the dynamic SSSP batch update on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl dsssp|reference] [--workload NAME]

Default workload (rmat22): RMAT(a=.57, b=.19, c=.19, d=.05) scale 22, 33,554,432 distinct
undirected edges, int32 weights U[1,100], source = highest-degree vertex; one batch of 1,000,000
changes (500,000 insertions of new pairs drawn from the same RMAT distribution, 500,000
deletions sampled without replacement from the edges).  Seeded synthetic inputs.

A step applies the batch to the resident graph and tree.  Between steps the graph and tree are
restored from a device snapshot and a 256 MB buffer is written (L2 flush); neither is timed.
  value  = changes applied / device time of the update (CUDA events on the launching stream,
           batch records already in HBM), summed over all ranks' work / max over ranks
  e2e    = the same metric through the public C ABI with host buffers: dsssp_apply_batch
           from pinned host memory + dsssp_tree_read into pinned host memory, host clock
On one GPU the default line also carries the other halves of the metric, measured after the
headline on the same GPU:
  batched_over_plain      the batch256 workload: 256 graphs' batches in one launch sequence of a
                          pooled store against the same batches applied one by one (device time)
  serve                   the serve workload: capacity, then p50/p99 latency and throughput at
                          offered loads of 0.25-1.1 x capacity (continuous batching)
  served_over_one_by_one  the saturated serving stream applied one request at a time by the
                          plain update, against the served capacity on the same stream
(--headline-only skips them.)
Multi-GPU (torchrun): the update of one graph does not shard, so every rank runs an
independent replica (weak scaling, no collective on the data path).

--impl reference times the reference's CPU path -- a full sequential recompute
(seqSSSPwithDist_undir.cpp's Dijkstra) of the updated graph -- on the host, rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

WORKLOADS = {
    "serve": dict(kind="serve", rmat_scale=24, rmat_m=134_217_728, tenants=32, tnlo=5.0, tnhi=6.30103, degree=8,
                  wlo=1, whi=100, blo=1.0, bhi=5.0, loads=(0.25, 0.5, 0.75, 0.9, 1.1), requests=2000, checked=4),
    "batch256": dict(kind="batch", count=256, nlo=3.0, nhi=6.0, degree=8, wlo=1, whi=100, flo=-3.0, fhi=-1.0,
                     slack_pct=50, slack_min=16),
    "rmat22": dict(kind="rmat", scale=22, m=33_554_432, wlo=1, whi=100, n_ins=500_000, n_del=500_000),
    "er10k": dict(kind="er", n=10_000, m=50_000, wlo=1, whi=100, n_ins=500, n_del=500),
    "grid4096": dict(kind="grid", rows=4096, cols=4096, remove=0.05, diag=167_772, wlo=1, whi=1000,
                     n_ins=25_000, n_del=75_000),
    # smaller cases of the same kernels, for profiler captures that must stay within a few GB
    "grid2048": dict(kind="grid", rows=2048, cols=2048, remove=0.05, diag=41_943, wlo=1, whi=1000,
                     n_ins=6_250, n_del=18_750),
    "batch64": dict(kind="batch", count=64, nlo=3.0, nhi=5.5, degree=8, wlo=1, whi=100, flo=-3.0, fhi=-1.0,
                    slack_pct=50, slack_min=16),
}


def describe(name: str) -> dict:
    w = WORKLOADS[name]
    if w["kind"] == "serve":
        return {"workload": name,
                "graph": f"resident RMAT(.57,.19,.19,.05) scale {w['rmat_scale']} with {w['rmat_m']} edges + "
                         f"{w['tenants']} Erdos-Renyi tenants, n log-uniform in [1e{w['tnlo']:.0f}, 2e6], "
                         f"average degree {w['degree']}, w U[{w['wlo']},{w['whi']}]",
                "batch": f"Poisson arrivals, sizes log-uniform in [1e{w['blo']:.0f}, 1e{w['bhi']:.0f}], 50% insertions",
                "loads": list(w["loads"]), "requests_per_load": w["requests"], "seed": 0}
    if w["kind"] == "batch":
        return {"workload": name, "graphs": w["count"],
                "graph": f"Erdos-Renyi, n log-uniform in [1e{w['nlo']:.0f}, 1e{w['nhi']:.0f}], average degree "
                         f"{w['degree']}, w U[{w['wlo']},{w['whi']}], source vertex 0 of each",
                "batch": f"per graph ceil(f*m), f log-uniform in [1e{w['flo']:.0f}, 1e{w['fhi']:.0f}], 50% insertions",
                "seed": 0}
    if w["kind"] == "rmat":
        g = f"RMAT(.57,.19,.19,.05) scale {w['scale']}, {w['m']} edges, w U[{w['wlo']},{w['whi']}], src = max degree"
    elif w["kind"] == "er":
        g = f"Erdos-Renyi n={w['n']} m={w['m']}, w U[{w['wlo']},{w['whi']}], src 0"
    else:
        g = (f"{w['rows']}x{w['cols']} grid, {w['remove']:.0%} of 4-neighbour edges removed, "
             f"{w['diag']} diagonals, w U[{w['wlo']},{w['whi']}], src 0")
    return {"workload": name, "graph": g, "batch": w["n_ins"] + w["n_del"], "insertions": w["n_ins"],
            "deletions": w["n_del"], "seed": 0}


def make_inputs(name: str):
    import dynamicssspv2_gb300 as D

    w = WORKLOADS[name]
    if w["kind"] == "rmat":
        n = 1 << w["scale"]
        u, v, wt = D.gen_rmat(w["scale"], w["m"], 0.57, 0.19, 0.19, w["wlo"], w["whi"], seed=0)
        src = D.max_degree_vertex(n, u, v)
        ch = D.gen_changes(n, u, v, wt, w["n_ins"], w["n_del"], D.INS_RMAT, w["scale"], 0.57, 0.19, 0.19,
                           w["wlo"], w["whi"], seed=1)
    elif w["kind"] == "er":
        n = w["n"]
        u, v, wt = D.gen_er(n, w["m"], w["wlo"], w["whi"], seed=0)
        src = 0
        ch = D.gen_changes(n, u, v, wt, w["n_ins"], w["n_del"], seed=1, wlo=w["wlo"], whi=w["whi"])
    else:
        n = w["rows"] * w["cols"]
        u, v, wt = D.gen_grid(w["rows"], w["cols"], w["remove"], w["diag"], w["wlo"], w["whi"], seed=0)
        src = 0
        ch = D.gen_changes(n, u, v, wt, w["n_ins"], w["n_del"], D.INS_LOCAL, w["cols"], 2.0, 0, 0, w["wlo"],
                           w["whi"], seed=1)
    return n, u, v, wt, src, ch


# ---- distributed plumbing (torchrun: one process per GPU) ------------------------------------

class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist

            backend = "nccl" if os.environ.get("DSSSP_BENCH_BACKEND", "nccl") == "nccl" else "gloo"
            if backend == "nccl":
                import torch

                torch.cuda.set_device(self.local)
            dist.init_process_group(backend=backend)
            self.pg = dist
            self.backend = backend

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch

        dev = torch.device("cuda", self.local) if self.backend == "nccl" else torch.device("cpu")
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


def whole_job_rate(dist: "Dist", batch: int, steps: int, local_seconds: float) -> tuple[float, float]:
    """Replicas: every rank applies `steps` batches of `batch` changes; the job's time is the
    slowest rank's.  Returns (change-edges/s over all ranks, max seconds)."""
    t_max = dist.max(local_seconds)
    return dist.world * batch * steps / t_max, t_max


# ---- clocks ---------------------------------------------------------------------------------

class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None

    def __enter__(self):
        if os.environ.get("DSSSP_BENCH_NO_CLOCKS"):
            return self
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in getattr(self, "lines", []):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---- helpers ----------------------------------------------------------------------------------

def measured_peak_hbm() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return 6800.0, "fallback"


def profiled_value(stem: str, workload: str, key: str):
    """A `key=value` figure from the committed ncu summary profiles/<stem>_<workload>.txt."""
    p = ROOT / "profiles" / f"{stem}_{workload}.txt"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith(key + "="):
            try:
                return float(line.split("=", 1)[1])
            except ValueError:
                return None
    return None


def profiled_traffic(workload: str):
    """dram bytes per launch of the update kernel from the committed ncu summary, if any."""
    return profiled_value("k_update", workload, "dram_bytes_per_launch")


def front_roofline(workload: str, stats, peak: float) -> dict:
    """The batch front kernels' DRAM bandwidth: ncu bytes per launch (committed summary) over
    the live CUDA-event time of each kernel.  They are random-access bound, so this shows how
    close they run to the HBM, next to the update kernel's algorithmic-byte roofline."""
    out = {}
    for name, field in (("k_delete", "t_delete_ms"), ("k_append", "t_append_ms")):
        ms = statistics.mean(getattr(s, field) for s in stats)
        traffic = profiled_value("front_kernels", workload, f"{name}_dram_bytes_per_launch")
        rate = traffic / (ms * 1e-3) / 1e9 if traffic and ms > 0 else None
        out[name] = {"ms_per_launch": ms, "traffic": traffic, "achieved_dram_gbs": rate,
                     "frac_dram": rate / peak if rate else None}
    return out


def cpu_recompute(n, u, v, w, ch, src, reps=1):
    """The reference's CPU path: a full sequential Dijkstra of the updated graph (one core)."""
    from oracle import pyoracle as O

    g = O.updated_graph(n, u, v, w, ch)
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        O.dijkstra(n, g, src)
        times.append(time.perf_counter() - t0)
    return times


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# ---- arms -------------------------------------------------------------------------------------

def make_inputs_cpu(name: str):
    """The workload's inputs from the oracle's restatement of the generators (bit-identical to
    make_inputs, which uses the library's): the CPU reference arm loads no product library."""
    from oracle import pyoracle as O

    w = WORKLOADS[name]
    if w["kind"] == "rmat":
        n = 1 << w["scale"]
        u, v, wt = O.gen_rmat(w["scale"], w["m"], 0.57, 0.19, 0.19, w["wlo"], w["whi"], 0)
        src = O.max_degree_vertex(n, u, v)
        ch = O.gen_changes(n, u, v, wt, w["n_ins"], w["n_del"], 1, w["scale"], 0.57, 0.19, 0.19, w["wlo"], w["whi"], 1)
    elif w["kind"] == "er":
        n = w["n"]
        u, v, wt = O.gen_er(n, w["m"], w["wlo"], w["whi"], 0)
        src = 0
        ch = O.gen_changes(n, u, v, wt, w["n_ins"], w["n_del"], 0, 0, 0.0, 0.0, 0.0, w["wlo"], w["whi"], 1)
    else:
        raise ValueError(f"{name}: no CPU restatement of this workload's generator")
    return n, u, v, wt, src, ch


def run_reference(args, dist: Dist) -> int:
    if dist.rank != 0:
        return 0
    if WORKLOADS[args.workload]["kind"] not in ("rmat", "er"):
        print(json.dumps({"impl": "reference", "unavailable": f"the CPU reference arm runs the rmat22 and er10k "
                          f"workloads (their generators are restated on the CPU side); not {args.workload}"}))
        return 0
    n, u, v, w, src, ch = make_inputs_cpu(args.workload)
    batch = len(ch)
    for _ in range(args.warmup):
        cpu_recompute(n, u, v, w, ch, src)
    times = []
    for _ in range(args.steps):
        times += cpu_recompute(n, u, v, w, ch, src)
    total = sum(times)
    value = batch * len(times) / total
    line = {
        "impl": "reference",
        "metric": "change-edges/s (batch update, exact distances)",
        "value": value,
        "unit": "change-edges/s",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * total / len(times),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int64",
        "data": "synthetic",
        "config": describe(args.workload),
        "cpu_baseline": {"value": value, "unit": "change-edges/s", "cores": 1, "kind": "port",
                         "sample": "one full sequential recompute (oracle restatement of "
                                   "seqSSSPwithDist_undir.cpp djk) of the updated graph per step, "
                                   f"1 of {host_cores()} host cores (the algorithm is sequential)"},
        "e2e": {"value": value, "unit": "change-edges/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def pipelined_e2e(D, g, ch, h_ch, h_dist32_after, reset, sptr, pairs: int = 5) -> dict:
    """End to end over a stream of batches through the C ABI: the batch B and its inverse
    (B's insertions deleted, its deletions inserted again: a valid batch of the same size and
    mix) alternate, each uploaded from pinned host memory and applied (dsssp_apply_batch), each
    updated tree read back as int32 parents and uint32 distances (dsssp_tree_read32_async), the
    copy overlapping the next batch's upload and kernels.  Checked: after B the distances are
    those of B alone (the e2e leg's last read), after B and its inverse those of the start.
    Every batch adds 2 x 500k adjacency entries while its deletions only tombstone theirs, so
    rows outgrow their slack and, within about ten steps, the spare region: the repack that
    follows (a full compaction) is part of the timed stream.  apply_ms shows each step.
    Returns a dict (see its keys)."""
    import ctypes as C

    import torch

    n = g.n
    inv = ch.copy()
    live = (ch["op"] == 0) | (ch["op"] == 1)
    inv["op"][live] = 1 - ch["op"][live]
    h_inv = torch.from_numpy(inv.view(np.uint8).copy()).pin_memory()
    trees = [(torch.empty(n, dtype=torch.int32).pin_memory(), torch.empty(n, dtype=torch.int32).pin_memory())
             for _ in range(2)]
    after_b = h_dist32_after.numpy().view(np.uint32).copy()
    reset()
    start = g.tree_read32()[1]
    steps = 2 * pairs
    st = D.Stats()
    apply_ms, repacks = [], 0
    t0 = time.perf_counter()
    for i in range(steps):
        rec = h_ch if i % 2 == 0 else h_inv
        ta = time.perf_counter()
        D._check(D._lib.dsssp_apply_batch(g.handle, rec.data_ptr(), len(ch), sptr, C.byref(st)), "apply_batch")
        apply_ms.append(round(1e3 * (time.perf_counter() - ta), 3))
        repacks += st.repacks
        p, d = trees[i % 2]
        D._check(D._lib.dsssp_tree_read32_async(g.handle, p.data_ptr(), d.data_ptr()), "tree_read32_async")
    D._check(D._lib.dsssp_tree_read_wait(g.handle), "tree_read_wait")
    dt = time.perf_counter() - t0
    exact = (np.array_equal(trees[0][1].numpy().view(np.uint32), after_b)
             and np.array_equal(trees[1][1].numpy().view(np.uint32), start))
    reset()
    return {"value": steps * len(ch) / dt, "unit": "change-edges/s", "ms_per_step": 1e3 * dt / steps, "steps": steps,
            "h2d_bytes_per_step": int(ch.nbytes), "d2h_bytes_per_step": n * 8, "exact": bool(exact),
            "apply_ms": apply_ms, "repacks": repacks,
            "timed": "host clock over all steps",
            "pattern": "B and its inverse alternating on the resident graph; each step uploads its records and reads "
                       "back the whole updated tree (parent int32 + dist uint32), the read overlapping the next step"}


def run_engine(args, dist: Dist) -> int:
    import dynamicssspv2_gb300 as D

    dev = dist.local
    n, u, v, w, src, ch = make_inputs(args.workload)
    batch = len(ch)
    opts = D.default_opts(device=dev)
    for key, val in json.loads(os.environ.get("DSSSP_BENCH_OPTS", "{}")).items():
        setattr(opts, key, val)
    g = D.Graph(n, u, v, w, opts)
    g.tree_compute(src)
    g.snapshot()

    import torch

    torch.cuda.set_device(dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{dev}")
    d_ch = torch.from_numpy(ch.view(np.int32).reshape(-1)).to(f"cuda:{dev}")
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream

    # pinned host buffers for the end-to-end leg
    nbytes = ch.nbytes
    h_ch = torch.from_numpy(ch.view(np.uint8).copy()).pin_memory()
    h_par = torch.empty(n, dtype=torch.int32).pin_memory()
    h_dist = torch.empty(n, dtype=torch.int64).pin_memory()
    h_dist32 = torch.empty(n, dtype=torch.int32).pin_memory()  # uint32 distances, same width
    h_vtx = torch.empty(n, dtype=torch.int32).pin_memory()
    import ctypes as C

    def reset():
        g.restore(sptr)
        flush.fill_(1)
        torch.cuda.synchronize(dev)

    def device_step():
        g.apply_batch_async(d_ch.data_ptr(), batch, sptr)
        return g.batch_finish()

    def e2e_step():  # the batch and the whole updated tree (parent int32, dist uint32)
        t0 = time.perf_counter()
        st = D.Stats()
        D._check(D._lib.dsssp_apply_batch(g.handle, h_ch.data_ptr(), batch, sptr, C.byref(st)), "apply_batch")
        D._check(D._lib.dsssp_tree_read32(g.handle, h_par.data_ptr(), h_dist32.data_ptr()), "tree_read32")
        return time.perf_counter() - t0, st

    def e2e_read64_step():  # the same with 64-bit distances (dsssp_tree_read)
        t0 = time.perf_counter()
        st = D.Stats()
        D._check(D._lib.dsssp_apply_batch(g.handle, h_ch.data_ptr(), batch, sptr, C.byref(st)), "apply_batch")
        D._check(D._lib.dsssp_tree_read(g.handle, h_par.data_ptr(), h_dist.data_ptr()), "tree_read")
        return time.perf_counter() - t0, st

    def e2e_delta_step():  # the same batch, reading back only the entries it may have changed
        t0 = time.perf_counter()
        st = D.Stats()
        cnt = C.c_int64()
        D._check(D._lib.dsssp_apply_batch(g.handle, h_ch.data_ptr(), batch, sptr, C.byref(st)), "apply_batch")
        D._check(D._lib.dsssp_tree_read_changed(g.handle, h_vtx.data_ptr(), h_par.data_ptr(), h_dist.data_ptr(), n,
                                                C.byref(cnt)), "tree_read_changed")
        return time.perf_counter() - t0, cnt.value

    clk = ClockSampler(dev).__enter__()
    if clk.proc:
        time.sleep(1.0)  # let nvidia-smi come up before any timed work
    for _ in range(args.warmup):
        reset()
        device_step()

    # timed: K steps, device time from CUDA events recorded by the library on the stream
    dist.barrier()
    torch.cuda.synchronize(dev)
    stats = []
    launches0 = D.launch_count()
    for _ in range(args.steps):
        reset()
        stats.append(device_step())
    launches = D.launch_count() - launches0
    torch.cuda.synchronize(dev)
    dist.barrier()
    # the resets between steps launch restore copies and the flush (not library kernels);
    # library kernels per step: prepare, delete, append, update
    t_steps = [s.t_total_ms for s in stats]
    value, t_max = whole_job_rate(dist, batch, args.steps, sum(t_steps) * 1e-3)

    # end-to-end through the C ABI with host buffers (median over the steps: host-side
    # copies see more run-to-run noise than the device)
    e2e_times, read64_times, delta_times, delta_counts = [], [], [], []
    for _ in range(max(5, min(args.steps, 20))):
        reset()
        dt, _ = e2e_step()
        e2e_times.append(dt)
    for _ in range(max(5, min(args.steps, 20))):
        reset()
        dt, _ = e2e_read64_step()
        read64_times.append(dt)
    for _ in range(max(5, min(args.steps, 20))):
        reset()
        dt, cnt = e2e_delta_step()
        delta_times.append(dt)
        delta_counts.append(cnt)
    pipe = pipelined_e2e(D, g, ch, h_ch, h_dist32, reset, sptr)
    clk.__exit__(None, None, None)
    e2e_value, e2e_t = whole_job_rate(dist, batch, 1, statistics.median(e2e_times))
    read64_value, read64_t = whole_job_rate(dist, batch, 1, statistics.median(read64_times))

    # the front kernels one by one: timing level 2 records events between them, in a few more
    # batches after the timed ones, so the headline steps carry none of their cost
    opts.timing = 2
    g.set_opts(opts)
    front_stats = []
    for _ in range(5):
        reset()
        front_stats.append(device_step())
    delta_value, delta_t = whole_job_rate(dist, batch, 1, statistics.median(delta_times))

    # roofline of the dominant kernel (the persistent update kernel)
    upd_ms = statistics.mean(s.t_update_ms for s in stats)
    upd_bytes = statistics.mean(s.bytes_alg_update for s in stats)
    eng_bytes = statistics.mean(s.bytes_engine_update for s in stats)
    peak, peak_kind = measured_peak_hbm()
    achieved = upd_bytes / (upd_ms * 1e-3) / 1e9
    s0 = stats[-1]

    cpu = None
    if dist.rank == 0 and not args.no_cpu_baseline:
        ct = cpu_recompute(n, u, v, w, ch, src, reps=1)[0]
        cpu = {"value": batch / ct, "unit": "change-edges/s", "cores": 1, "kind": "port",
               "sample": f"one full sequential recompute (oracle restatement of seqSSSPwithDist_undir.cpp djk) "
                         f"of the updated graph, {ct:.2f} s, 1 of {host_cores()} host cores"}
    clocks = clk.summary()
    g.close()
    if dist.rank != 0:
        dist.close()
        return 0
    cfg = describe(args.workload)
    cfg.update({"parallelism": f"replicas x{dist.world}", "l2": "graph restore (>1 GB written) + 256 MB flush "
                "between timed steps", "timed": "sum of per-step CUDA-event intervals around the batch kernels",
                "clocks_window": "nvidia-smi every 50 ms from 1 s before warm-up to the end of the e2e leg",
                "opts": {k: getattr(opts, k) for k, _ in D.Opts._fields_}})
    line = {
        "metric": "change-edges/s (batch update, exact distances)",
        "value": value,
        "unit": "change-edges/s",
        "n_gpus": dist.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * t_max / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int32",
        "data": "synthetic",
        "config": cfg,
        "e2e": {"value": e2e_value, "unit": "change-edges/s", "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": n * (4 + 4) + 320, "ms_per_step": 1e3 * e2e_t,
                "ms_all_steps": [round(1e3 * t, 4) for t in e2e_times], "timed": "host clock per step, median",
                "result": "the whole updated tree (dsssp_tree_read32: parent int32 + dist uint32 per vertex, "
                          "the widths of the reference's RT_Vertex)",
                "read64": {"value": read64_value, "ms_per_step": 1e3 * read64_t, "d2h_bytes_per_step": n * (4 + 8) + 320,
                           "result": "the same tree with int64 distances (dsssp_tree_read)"},
                "host_link": "pinned host buffers; H2D and D2H each run near 190 GB/s on this box"},
        "e2e_pipelined": pipe,
        "e2e_changed": {"value": delta_value, "unit": "change-edges/s", "h2d_bytes_per_step": nbytes,
                        "d2h_bytes_per_step": int(statistics.median(delta_counts)) * (4 + 4 + 8) + 8 + 320,
                        "ms_per_step": 1e3 * delta_t, "changed_vertices": int(statistics.median(delta_counts)),
                        "timed": "host clock per step, median",
                        "result": "the entries the batch may have changed (dsssp_tree_read_changed: vertex, "
                                  "parent, dist), which rebuild the updated tree from the previous one"},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": profiled_traffic(args.workload),
                     "kernel": "k_update", "peak_kind": peak_kind, "ms_per_launch": upd_ms,
                     "alg_bytes_per_launch": upd_bytes,
                     "alg_model": "per-unit byte model: 16 B per cut-off vertex + 4 B per child, 20 B per frontier "
                                  "vertex (pulls included) + 16 B per scanned edge, 12 B per lowering atomic",
                     "engine_bytes_per_launch": eng_bytes,
                     "achieved_engine_count": eng_bytes / (upd_ms * 1e-3) / 1e9,
                     "front_kernels": front_roofline(args.workload, front_stats, peak)},
        "cpu_baseline": cpu,
        "clocks": clocks,
        "detail": {
            "rounds": s0.rounds, "advances": s0.advances, "frontier_total": s0.frontier_total, "edges_relaxed": s0.edges_relaxed,
            "edges_inval": s0.edges_inval, "invalidated": s0.n_invalidated, "roots": s0.n_roots,
            "inv_levels": s0.inv_levels, "pj_passes": s0.pj_passes, "updates": s0.updates,
            "repacks": sum(s.repacks for s in stats), "t_step1_ms": s0.t_step1_ms, "t_update_ms": s0.t_update_ms,
            "t_inval_ms": s0.t_inval_ms, "t_relax_ms": s0.t_relax_ms,
            "affected_edges_per_s": (s0.edges_relaxed + s0.edges_inval) / (s0.t_total_ms * 1e-3),
            "step_ms": t_steps,
        },
    }
    if args.workload == "rmat22" and dist.world == 1 and not args.headline_only:
        line.update(extra_workloads(args, dist))
    dist.close()
    print(json.dumps(line), flush=True)
    return 0


def extra_workloads(args, dist: Dist) -> dict:
    """The batching and serving halves of the metric, run after the headline on the same GPU
    (one at a time; each frees its device memory before the next): batched over plain on the
    256-graph workload, and p50/p99 under load with the served-over-one-by-one ratio on the
    serving workload."""
    out = {}
    steps, warmup = max(3, min(args.steps, 10)), max(3, min(args.warmup, 3))
    b = batching_summary("batch256", steps, warmup, dist)
    out["batched_over_plain"] = {
        "ratio": b["batched_over_plain"], "workload": "batch256",
        "batched": {"value": b["value"], "unit": b["unit"], "ms_per_step": b["ms_per_step"],
                    "wall_ms_per_step": b["batched_wall_ms_per_step"]},
        "plain": b["plain"], "steps": b["steps"], "warmup": b["warmup"],
        "mismatched_distances": b["mismatched_distances"], "gpu_launches": b["gpu_launches"],
        "graphs": b["config"]["graphs"], "vertices": b["config"]["vertices"], "edges": b["config"]["edges"],
        "changes": b["config"]["changes"], "autotuned": b["config"]["autotuned"], "clocks": b["clocks"],
        "timed": "device time (CUDA events) of the batch kernels: one union batch through one launch sequence of "
                 "the pooled store, against the 256 batches applied one by one to graph stores of their own; "
                 "restore + 256 MB L2 flush before each update untimed"}
    s = serving_summary("serve", dist)
    keep = ("offered_load", "offered_requests_per_s", "requests", "served", "changes", "change_edges_per_s",
            "p50_ms", "p99_ms", "mean_ms", "mean_requests_per_epoch", "certificate_violations")
    out["serve"] = {
        "workload": "serve", "capacity_change_edges_per_s": s["capacity"]["change_edges_per_s"],
        "loads": [{k: ld[k] for k in keep} for ld in s["loads"]],
        "admitted": s["config"]["admitted"], "vertices": s["config"]["vertices"], "edges": s["config"]["edges"],
        "checked_tenants": s["checked_tenants"], "mismatched_distances": s["mismatched_distances"],
        "clocks": s["clocks"], "timed": s["config"]["timed"]}
    out["served_over_one_by_one"] = s["one_by_one"]
    return out


def make_batch_inputs(name: str):
    """The batching workload: many independent graphs, each with its own batch."""
    from concurrent.futures import ThreadPoolExecutor

    import dynamicssspv2_gb300 as D

    w = WORKLOADS[name]
    rng = np.random.default_rng(0)
    ns = np.round(10 ** rng.uniform(w["nlo"], w["nhi"], w["count"])).astype(np.int64)
    fs = 10 ** rng.uniform(w["flo"], w["fhi"], w["count"])

    def one(i):
        n = int(ns[i])
        m = n * w["degree"] // 2
        u, v, wt = D.gen_er(n, m, w["wlo"], w["whi"], seed=1000 + i)
        k = max(2, int(np.ceil(fs[i] * m)))
        ch = D.gen_changes(n, u, v, wt, k // 2, k - k // 2, seed=2000 + i, wlo=w["wlo"], whi=w["whi"])
        return n, u, v, wt, ch

    with ThreadPoolExecutor(4) as ex:
        return list(ex.map(one, range(w["count"])))


def run_batching(args, dist: Dist) -> int:
    line = batching_summary(args.workload, args.steps, args.warmup, dist)
    dist.close()
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def batching_summary(workload: str, steps: int, warmup: int, dist: Dist) -> dict:
    """Many graphs: one batch per graph applied one by one with the plain update, against all
    of them together in one launch sequence on a pooled graph store (autotuned)."""
    import tempfile

    import torch

    import dynamicssspv2_gb300 as D
    from dynamicssspv2_gb300.autotune import Autotuner
    from dynamicssspv2_gb300.pool import GraphPool

    dev = dist.local
    torch.cuda.set_device(dev)
    t0 = time.perf_counter()
    items = make_batch_inputs(workload)
    t_gen = time.perf_counter() - t0
    total_changes = sum(len(it[4]) for it in items)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{dev}")

    # plain: one graph store per graph, batches applied one after another
    plain = []
    wl = WORKLOADS[workload]
    slack = {"slack_pct": wl["slack_pct"], "slack_min": wl["slack_min"]}
    for n, u, v, wt, ch in items:
        g = D.Graph(n, u, v, wt, device=dev, **slack)
        g.tree_compute(0)
        g.snapshot()
        d = torch.from_numpy(ch.view(np.int32).reshape(-1)).to(f"cuda:{dev}")
        plain.append((g, d, len(ch)))
    # batched: all graphs in one pool, all batches in one union batch
    pool = GraphPool([(n, u, v, wt) for n, u, v, wt, _ in items], device=dev, **slack)
    pool.tree_compute([0] * len(items))
    union = pool.union_batch([(i, it[4]) for i, it in enumerate(items)])
    d_union = torch.from_numpy(union.view(np.int32).reshape(-1)).to(f"cuda:{dev}")
    cache = os.environ.get("DSSSP_AUTOTUNE_CACHE") or os.path.join(tempfile.gettempdir(), "dsssp_autotune.txt")
    tuned = Autotuner(cache).tune(pool.graph, union)
    pool.graph.snapshot()

    def flush_l2():
        flush.fill_(1)
        torch.cuda.synchronize(dev)

    def plain_pass():
        t_dev, t_wall = 0.0, 0.0
        for g, d, k in plain:
            g.restore()
            flush_l2()
            w0 = time.perf_counter()
            g.apply_batch_async(d.data_ptr(), k)
            st = g.batch_finish()
            t_wall += time.perf_counter() - w0
            t_dev += st.t_total_ms * 1e-3
        return t_dev, t_wall

    def pooled_pass():
        pool.graph.restore()
        flush_l2()
        w0 = time.perf_counter()
        pool.graph.apply_batch_async(d_union.data_ptr(), len(union))
        st = pool.graph.batch_finish()
        return st.t_total_ms * 1e-3, time.perf_counter() - w0, st

    for _ in range(warmup):
        plain_pass()
        pooled_pass()
    clk = ClockSampler(dev).__enter__()
    if clk.proc:
        time.sleep(1.0)
    dist.barrier()
    pd, pw, bd, bw, stats, repacks = 0.0, 0.0, 0.0, 0.0, None, 0
    launches0 = D.launch_count()
    for _ in range(steps):
        a, b = plain_pass()
        pd += a
        pw += b
        c, d_, stats = pooled_pass()
        bd += c
        bw += d_
        repacks += stats.repacks
    launches = D.launch_count() - launches0
    dist.barrier()
    clk.__exit__(None, None, None)
    # exactness spot check: pooled result of every graph == its plain result
    mismatches = 0
    for i, (g, _, _) in enumerate(plain):
        p_plain, d_plain = g.tree_read()
        p_pool, d_pool = pool.tree_read(i)
        mismatches += int((d_plain != d_pool).sum())
    value, t_max = whole_job_rate(dist, total_changes, steps, bd)
    plain_value, _ = whole_job_rate(dist, total_changes, steps, pd)
    for g, _, _ in plain:
        g.close()
    pool.close()
    cfg = describe(workload)
    cfg.update({"vertices": int(sum(it[0] for it in items)), "edges": int(sum(len(it[1]) for it in items)),
                "changes": int(total_changes), "autotuned": tuned["opts"], "autotune_key": tuned["key"],
                "timed": "sum of CUDA-event intervals of the batch kernels; graph restore + 256 MB flush "
                         "before each update untimed", "parallelism": f"replicas x{dist.world}",
                "slack": slack})
    line = {
        "metric": "change-edges/s (batched: all graphs' batches in one launch sequence)",
        "value": value,
        "unit": "change-edges/s",
        "n_gpus": dist.world,
        "steps": steps,
        "warmup": warmup,
        "ms_per_step": 1e3 * t_max / steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int32",
        "data": "synthetic",
        "config": cfg,
        "plain": {"value": plain_value, "unit": "change-edges/s", "ms_per_step": 1e3 * pd / steps,
                  "wall_ms_per_step": 1e3 * pw / steps},
        "batched_over_plain": value / plain_value,
        "batched_wall_ms_per_step": 1e3 * bw / steps,
        "mismatched_distances": mismatches,
        "pooled_repacks": repacks,
        "gpu_launches": launches,
        "detail": {"rounds": stats.rounds, "inv_levels": stats.inv_levels, "invalidated": stats.n_invalidated,
                   "edges_relaxed": stats.edges_relaxed, "t_step1_ms": stats.t_step1_ms,
                   "t_update_ms": stats.t_update_ms, "setup_gen_s": t_gen},
        "clocks": clk.summary(),
    }
    return line


def run_serving(args, dist: Dist) -> int:
    line = serving_summary(args.workload, dist)
    dist.close()
    if dist.rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def one_by_one(tenants, streams, dev: int, slack: dict):
    """The plain single-batch update on the same request streams: every tenant in a graph
    store of its own, each request's batch applied alone from host memory through the C ABI
    (dsssp_apply_batch, which waits for the result).  streams = [(requests, timed)], applied
    in arrival order.  Returns (changes, seconds) of the timed streams and the tenants' final
    distances."""
    import dynamicssspv2_gb300 as D

    graphs = []
    for t in tenants:
        g = D.Graph(t.n, t.u, t.v, t.w, device=dev, **slack)
        g.tree_compute(t.src)
        graphs.append(g)
    changes, secs = 0, 0.0
    for reqs, timed in streams:
        for r in sorted(reqs, key=lambda r: r.arrival):
            a = np.ascontiguousarray(r.changes, D.CHANGE_DTYPE)
            t0 = time.perf_counter()
            graphs[r.tenant].apply_batch(a)
            dt = time.perf_counter() - t0
            if timed:
                changes += len(a)
                secs += dt
    dists = [g.tree_read()[1] for g in graphs]
    for g in graphs:
        g.close()
    return changes, secs, dists


def make_serve_tenants(workload: str):
    """The serving workload's tenants: the resident RMAT graph (source = its highest-degree
    vertex) and the Erdos-Renyi tenants (source 0), seeded."""
    from concurrent.futures import ThreadPoolExecutor

    import dynamicssspv2_gb300 as D
    from dynamicssspv2_gb300.serve import Tenant

    w = WORKLOADS[workload]
    rng = np.random.default_rng(0)
    ns = np.round(10 ** rng.uniform(w["tnlo"], w["tnhi"], w["tenants"])).astype(np.int64)

    def er(i):
        n = int(ns[i])
        u, v, wt = D.gen_er(n, n * w["degree"] // 2, w["wlo"], w["whi"], seed=3000 + i)
        return Tenant(f"er{i}", n, u, v, wt, src=0)

    with ThreadPoolExecutor(4) as ex:
        ers = list(ex.map(er, range(w["tenants"])))
    n_r = 1 << w["rmat_scale"]
    ru, rv, rw = D.gen_rmat(w["rmat_scale"], w["rmat_m"], 0.57, 0.19, 0.19, w["wlo"], w["whi"], seed=0)
    return [Tenant("rmat", n_r, ru, rv, rw, src=D.max_degree_vertex(n_r, ru, rv))] + ers


def serve_requests(workload: str, tenants, count: int, rate: float, seed: int):
    """count requests for random tenants: Poisson arrivals at `rate` per second (0 = all at
    once), batch sizes log-uniform in the workload's range, 50% insertions."""
    from dynamicssspv2_gb300.serve import Request, random_batch

    w = WORKLOADS[workload]
    g = np.random.default_rng(seed)
    sizes = np.round(10 ** g.uniform(w["blo"], w["bhi"], count)).astype(int)
    who = g.integers(0, len(tenants), count)
    arr = np.cumsum(g.exponential(1.0 / rate, count)) if rate else np.zeros(count)
    return [Request(int(t), float(a), random_batch(g, tenants[int(t)], int(sz), wlo=w["wlo"], whi=w["whi"]))
            for t, a, sz in zip(who, arr, sizes)]


class EdgeTracker:
    """Edge lists of some tenants, kept up to date with every request applied to them (the
    reference's batch semantics, through the oracle), for exactness checks after serving."""

    def __init__(self, tenants, which):
        self.tenants = tenants
        self.lines = {t: (tenants[t].u, tenants[t].v, tenants[t].w) for t in which}

    def track(self, reqs) -> None:
        from oracle import pyoracle as O

        for r in sorted(reqs, key=lambda r: r.arrival):
            if r.tenant in self.lines and not r.refused and r.error is None:
                lines = self.lines[r.tenant]
                _, kept = O.updated_graph(self.tenants[r.tenant].n, *lines, r.changes, return_kept=True)
                ins = r.changes[r.changes["op"] == 1]
                lu = np.concatenate([lines[0], ins["u"]]).astype(np.int32)
                lv = np.concatenate([lines[1], ins["v"]]).astype(np.int32)
                lw = np.concatenate([lines[2], ins["w"]]).astype(np.int32)
                keep = kept[: len(lu)].astype(bool)
                self.lines[r.tenant] = (lu[keep], lv[keep], lw[keep])


def serving_summary(workload: str, dist: Dist, plain_baseline: bool = True) -> dict:
    """Serving: resident tenants, Poisson request stream, continuous batching; capacity, then
    p50/p99 latency and throughput at several offered loads; exactness on sampled tenants.
    With plain_baseline the saturated request stream is also applied one request at a time by
    the plain update (a graph store per tenant), which gives the served-over-one-by-one ratio
    on the same stream and checks every tenant's distances against the served ones."""
    from dynamicssspv2_gb300.serve import Server, summarize
    from oracle import pyoracle as O

    w = WORKLOADS[workload]
    dev = dist.local
    t0 = time.perf_counter()
    tenants = make_serve_tenants(workload)
    t_gen = time.perf_counter() - t0

    def make_requests(count, rate, seed):
        return serve_requests(workload, tenants, count, rate, seed)

    slack = {"slack_pct": 50, "slack_min": 16}
    srv = Server(tenants, device=dev, **slack)
    # exactness bookkeeping for the smallest ER tenants: their edge lists follow every request
    checked = sorted(range(1, len(tenants)), key=lambda t: tenants[t].n)[: w["checked"]]
    tracker = EdgeTracker(tenants, checked)
    track, lines = tracker.track, tracker.lines

    clk = ClockSampler(dev).__enter__()
    warm = make_requests(2 * len(tenants), 0, 1)
    srv.serve(warm, realtime=False)
    track(warm)
    sat = make_requests(w["requests"], 0, 2)
    srv.serve(sat, realtime=False)
    track(sat)
    cap = summarize(sat)
    cap_rate = cap["served"] / cap["span_s"]
    plain = None
    if plain_baseline:
        served_d = [srv.tree(t)[1] for t in range(len(tenants))]
        ch, secs, obo_d = one_by_one(tenants, [(warm, False), (sat, True)], dev, slack)
        differ = sum(int((a != b).sum()) for a, b in zip(served_d, obo_d))
        del served_d, obo_d
        rate = ch / secs if secs > 0 else 0.0
        plain = {"value": rate, "unit": "change-edges/s", "requests": len(sat), "changes": int(ch),
                 "seconds": secs, "served_value": cap["change_edges_per_s"],
                 "ratio": cap["change_edges_per_s"] / rate if rate > 0 else None,
                 "distances_differing_from_served": differ,
                 "how": "the saturated request stream applied one request at a time by the plain update "
                        "(each tenant in a graph store of its own, dsssp_apply_batch from host memory, host "
                        "clock per call, summed), after the same warm-up requests; ratio = served capacity "
                        "over this rate"}
    loads = []
    for i, load in enumerate(w["loads"]):
        reqs = make_requests(w["requests"], load * cap_rate, 10 + i)
        srv.serve(reqs)
        track(reqs)
        st = summarize(reqs)
        st["offered_load"] = load
        st["offered_requests_per_s"] = load * cap_rate
        # device certificate of every tenant's tree after this load (untimed)
        st["certificate_violations"] = srv.validate()["violations"]
        loads.append(st)
    clk.__exit__(None, None, None)
    mism = 0
    for t in checked:
        p, d = srv.tree(t)
        n = tenants[t].n
        od, op = O.dijkstra(n, O.csr(n, *lines[t]), tenants[t].src)
        mism += int((od != d).sum())
    srv.close()
    cfg = describe(workload)
    cfg.update({"admitted": len(srv.admitted), "vertices": int(sum(t.n for t in tenants)),
                "edges": int(sum(len(t.u) for t in tenants)), "setup_gen_s": t_gen,
                "timed": "host clock from arrival to completion of each request (includes queueing, host batch "
                         "assembly, copies and the update)", "parallelism": "one pooled graph store, one GPU"})
    line = {
        "metric": "change-edges/s and p50/p99 per-batch latency under load (serving, continuous batching)",
        "value": cap["change_edges_per_s"],
        "unit": "change-edges/s",
        "n_gpus": dist.world,
        "steps": len(w["loads"]),
        "warmup": 1,
        "ms_per_step": cap["mean_ms"],
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int32",
        "data": "synthetic",
        "config": cfg,
        "capacity": cap,
        "one_by_one": plain,
        "loads": loads,
        "checked_tenants": len(checked),
        "mismatched_distances": mism,
        "clocks": clk.summary(),
    }
    return line


def run_once(args) -> int:
    """One batch of the workload, for a profiler: build the graph (or the pool), compute the tree,
    apply the batch once.  The update kernel's second launch is the batch's."""
    import dynamicssspv2_gb300 as D
    from dynamicssspv2_gb300.pool import GraphPool

    t0 = time.perf_counter()
    if WORKLOADS[args.workload]["kind"] == "batch":
        wl = WORKLOADS[args.workload]
        items = make_batch_inputs(args.workload)
        with GraphPool([(n, u, v, w) for n, u, v, w, _ in items], slack_pct=wl["slack_pct"],
                       slack_min=wl["slack_min"]) as pool:
            pool.tree_compute([0] * len(items))
            st = pool.apply([(i, it[4]) for i, it in enumerate(items)])
    else:
        n, u, v, w, src, ch = make_inputs(args.workload)
        with D.Graph(n, u, v, w) as g:
            g.tree_compute(src)
            st = g.apply_batch(ch)
    print(json.dumps({"workload": args.workload, "once": True, "t_total_ms": st.t_total_ms,
                      "t_update_ms": st.t_update_ms, "wall_s": time.perf_counter() - t0}), flush=True)
    return 0


def run_tour(args) -> int:
    """Every kernel of the library once, on an RMAT scale-20 graph (1M vertices, 8M edges: larger
    than the L2, a few hundred MB on the device): graph build, tree computation, a batch, the tree
    reads, the certificate, a batch whose rows grow into the spare region, compaction, a batch that
    repacks with overflowed entries, tree load, a pool graph added and removed, and the
    no-allocation entry point.  For a profiler's launch list; prints the host time of each step."""
    import torch

    import dynamicssspv2_gb300 as D
    from dynamicssspv2_gb300.pool import GraphPool
    from oracle import pyoracle as O

    steps = {}

    def step(name, fn):
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        steps[name] = round((time.perf_counter() - t0) * 1e3, 3)
        return r

    scale, m = 20, 8 << 20
    n = 1 << scale
    u, v, w = D.gen_rmat(scale, m, 0.57, 0.19, 0.19, 1, 100, seed=0)
    src = D.max_degree_vertex(n, u, v)
    ch = D.gen_changes(n, u, v, w, 100_000, 100_000, D.INS_RMAT, scale, 0.57, 0.19, 0.19, 1, 100, seed=1)
    g = step("graph_create", lambda: D.Graph(n, u, v, w, spare_pct=50))
    step("tree_compute", lambda: g.tree_compute(src))
    step("snapshot", g.snapshot)
    step("apply_batch", lambda: g.apply_batch(ch))
    step("tree_read", g.tree_read)
    step("tree_read_changed", g.tree_read_changed)
    step("validate", g.validate)
    # insertions around 64 vertices overflow their rows' slack: the rows move to the spare region
    rng = np.random.default_rng(3)
    hubs = rng.integers(0, n, 64)
    grow = D.make_changes(np.repeat(hubs, 500), rng.integers(0, n, 64 * 500), rng.integers(1, 101, 64 * 500),
                          np.ones(64 * 500))
    st = step("apply_batch_growing_rows", lambda: g.apply_batch(grow))
    steps["growth_overflow_entries"] = int(st.overflow_entries)
    step("compact", g.compact)
    parent, dist = g.tree_read()
    step("tree_load", lambda: g.tree_load(parent, dist))
    g.close()
    # no slack and no spare region: the batch's overflowed entries are folded in by a repack
    n2, m2 = 200_000, 800_000
    u2, v2, w2 = D.gen_er(n2, m2, 1, 100, seed=4)
    ch2 = D.gen_changes(n2, u2, v2, w2, 20_000, 20_000, seed=5)
    with D.Graph(n2, u2, v2, w2, slack_pct=0, slack_min=0, spare_pct=0) as g2:
        g2.tree_compute(0)
        st = step("apply_batch_repack", lambda: g2.apply_batch(ch2))
        steps["repacks"] = int(st.repacks)
    # a graph added to a pool's reserve and removed again
    with GraphPool([(n2, u2, v2, w2)], reserve_vertices=n2) as pool:
        pool.tree_compute([0])
        gi = step("pool_add_graph", lambda: pool.add_graph(n2, u2, v2, w2, src=7))
        step("pool_remove_graph", lambda: pool.remove_graph(gi))
    # the no-allocation entry point on caller-owned device buffers
    n3 = 60_000
    u3, v3, w3 = D.gen_er(n3, 4 * n3, 1, 100, seed=6)
    csr = O.csr(n3, u3, v3, w3)
    adj = np.ascontiguousarray(np.stack([csr.col, csr.wt], axis=1).astype(np.int32))
    d_off = torch.from_numpy(csr.off.astype(np.int64)).cuda()
    d_adj = torch.from_numpy(adj.reshape(-1)).cuda()
    d_par = torch.empty(n3, dtype=torch.int32, device="cuda")
    d_dist = torch.empty(n3, dtype=torch.int64, device="cuda")
    step("sssp_noalloc", lambda: D.sssp_noalloc(n3, len(csr.col), d_off.data_ptr(), d_adj.data_ptr(), 0,
                                                 d_par.data_ptr(), d_dist.data_ptr()))
    print(json.dumps({"workload": "tour", "graph": f"RMAT scale {scale}, {m} edges", "step_ms": steps,
                      "kernel_launches": D.launch_count()}), flush=True)
    return 0


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["dsssp", "reference"], default="dsssp")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + ["tour"], default="rmat22",
                    help="tour: every kernel of the library once (for a profiler's launch list)")
    ap.add_argument("--once", action="store_true", help="one batch of the workload, for a profiler")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--headline-only", action="store_true",
                    help="rmat22: skip the batching and serving workloads that the default line also carries")
    args = ap.parse_args()
    if args.workload == "tour":
        return run_tour(args)
    if args.once:
        return run_once(args)
    dist = Dist()
    if args.impl == "reference":
        if WORKLOADS[args.workload]["kind"] in ("batch", "serve"):
            if dist.rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the batching workload has no CPU reference "
                                  "arm; see the rmat22 workload"}))
            return 0
        return run_reference(args, dist)
    if WORKLOADS[args.workload]["kind"] == "batch":
        return run_batching(args, dist)
    if WORKLOADS[args.workload]["kind"] == "serve":
        return run_serving(args, dist)
    return run_engine(args, dist)


if __name__ == "__main__":
    sys.exit(main())
