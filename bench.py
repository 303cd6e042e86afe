#!/usr/bin/env python
"""Benchmark: tets/s of the per-tet implicit-arrangement path (stages a-d) on one GB300.

Default workload (the large degenerate implicit arrangement): tet5 grid with 129^3 vertices
(10,485,760 tets) over [-1,1]^3 and 32 FP64 functions: 8 planes (4 exact duplicates, 4 through grid
vertices), 8 spheres, 8 cylinders, 8 tori; seeded synthetic data.  --config mi runs the material
interface workload (65^3 vertices, 8 materials).

One step = sampling -> sign filter -> per-tet cut -> mesh extraction with vertex coordinates,
through the C ABI (ria_grid_implicit_arrangement); `value` is tets/s with the function
descriptors as the only input (the grid and its sampled values are produced on the device), timed
with CUDA events on the library's stream.  `e2e` goes through the reference-shaped host-buffer
entry points: ria_sample_functions (host points in, host values out, as the reference's
load_functions) and ria_compute_implicit_arrangement (host pts / tets / values in), then copies the
mesh (points, vertex records, faces) back; host<->device copies are inside its timed region.

--config batch runs the batched form: 4096 independent grids (vertices per axis uniform in 9..33,
2..24 functions of mixed kinds; about 2.3x10^8 tets) through ria_grid_batch, one pass of every stage
over all of them, and beside it the plain drop-in called once per grid (`per_problem_plain`).  Its
CPU baseline, and its --impl reference arm, run the CPU restatement over the first 256 grids with one
grid per process on every host core (the grids are independent).

--impl reference times the CPU restatement of the reference path (oracle/) on this host's cores over
the whole grid of the same workload (the reference itself depends on absent third-party libraries and
cannot be built).  Under torchrun only rank 0 runs it.  The GPU line's `cpu_baseline` is the same
restatement on one thread, the median of three passes over the whole grid.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)
PKG = "robust-implicit-surface-networks_gb300"

METRIC = "tets/s (arrangement+extract) on 1 GB300"

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one k_sample launch on the large
# degenerate workload, from one ncu capture of that launch
SAMPLE_TRAFFIC_WORKLOAD = "ia-degenerate-32func-res128"
SAMPLE_TRAFFIC = 4495360 + 521597184


def _peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples of SM clocks and throttle reasons while the timed region runs."""

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def workload(name, res=None):
    """The named workload; `res` (cubes per axis) overrides its grid size for profiling captures."""
    fns = importlib.import_module(PKG + ".functions")
    kw = {} if res is None else {"res": res}
    if name == "ia-degenerate":
        return fns.workload_ia_degenerate(**kw)
    if name == "mi":
        return fns.workload_mi(**kw)
    if name == "ia-small":
        return fns.workload_ia_small(**kw)
    raise SystemExit(f"unknown config {name}")


def _oracle_worker_init():
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle

    pyoracle.lib()
    importlib.import_module(PKG + ".functions")


def _oracle_worker_ready(_):
    time.sleep(0.05)
    return os.getpid()


def _oracle_problem(job):
    """One grid of the batch through the CPU restatement, stages a-d (a worker of cpu_batch)."""
    import pyoracle

    res, funcs, mode = job
    fns = importlib.import_module(PKG + ".functions")
    pts, tets = fns.generate_tet_mesh(res)
    fv = pyoracle.sample(funcs, pts)
    pyoracle.run(mode, pts, tets, fv)
    return len(tets)


def cpu_batch(probs, mode, n_problems=256, repeats=1):
    """The CPU restatement over the first n_problems grids of the batch, one process per host core
    (the grids are independent, so they spread over the cores without any exchange).  Returns
    per-repeat tets/s, the cores used and a description of the sample."""
    import multiprocessing as mp

    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle

    pyoracle.build()
    cores = os.cpu_count() or 1
    jobs = [(r, f, mode) for r, f in probs[:n_problems]]
    rates, n = [], 0
    with mp.get_context("spawn").Pool(cores, initializer=_oracle_worker_init) as pool:
        pool.map(_oracle_worker_ready, range(2 * cores), chunksize=1)  # every worker started
        for _ in range(repeats):
            t0 = time.perf_counter()
            n = sum(pool.map(_oracle_problem, jobs, chunksize=1))
            rates.append(n / (time.perf_counter() - t0))
    desc = (f"the first {len(jobs)} of {len(probs)} grids ({n} tets), stages a-d of the CPU restatement "
            f"(oracle/), one grid per process on {cores} cores")
    return rates, n, cores, desc


def max_over_ranks(x, dist, device):
    """The largest x over the ranks of the process group (x itself without one).  Every rank calls
    it at the same point: it is a collective."""
    if dist is None:
        return x
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference_batch(args, world):
    """The batched workload's CPU arm: every step is the bounded sample of cpu_batch."""
    fns = importlib.import_module(PKG + ".functions")
    wl = fns.workload_batch(n=args.batch_n)
    rates, n, cores, desc = cpu_batch(wl.problems, "ia", repeats=args.warmup + args.steps)
    per = statistics.median(rates[args.warmup:])
    line = {
        "impl": "reference", "metric": METRIC, "value": per, "unit": "tets/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": n / per * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": wl.name, "tets": wl.n_tets, "problems": len(wl.problems), "sample": desc},
        "cpu_baseline": {"value": per, "unit": "tets/s", "cores": cores, "kind": "port", "sample": desc},
        "e2e": {"value": per, "unit": "tets/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_batch(args, world, local):
    """The batched form against the plain drop-in called per problem."""
    import numpy as np
    import torch

    torch.cuda.set_device(local)
    fns = importlib.import_module(PKG + ".functions")
    pkg = importlib.import_module(PKG)
    pkg.build()
    L = pkg.load()
    wl = fns.workload_batch(n=args.batch_n)
    probs = wl.problems
    # the project's autotuner on a sample of the batch (the first 256 grids) chooses the cut's bins,
    # launch shapes and graph capture for this device before anything is timed
    tuned = None
    if args.tuning:
        pkg.set_tuning(dict(pkg.get_tuning(), **json.loads(args.tuning)))
    elif not args.no_tune:
        t0 = time.perf_counter()
        rec, best_s, dflt_s = pkg.autotune(probs[:256], reps=2)
        tuned = {"record": rec, "sample_problems": min(256, len(probs)), "sample_best_ms": best_s * 1e3,
                 "sample_default_ms": dflt_s * 1e3, "tuner_wall_s": time.perf_counter() - t0}
    for _ in range(args.warmup):
        pkg.grid_batch(probs).close()
    launches0 = int(L.ria_kernel_launches())
    dev_ms, stage = [], {"sample": [], "filter": [], "cut": [], "extract": []}
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            L.ria_lookup_cache_clear()
            m = pkg.grid_batch(probs)
            tm = m.timings
            dev_ms.append(tm["total"] * 1e3)
            for k in stage:
                stage[k].append(tm[k] * 1e3)
            st = m.stats
            m.close()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    launches = int(L.ria_kernel_launches()) - launches0
    ms = statistics.mean(dev_ms)
    value = wl.n_tets / (ms * 1e-3)
    # end to end: descriptors in, the whole mesh of every problem back on the host
    e2e_t = []
    d2h = 0
    for it in range(0 if args.no_e2e else 1 + args.steps):
        L.ria_lookup_cache_clear()
        t0 = time.perf_counter()
        m = pkg.grid_batch(probs)
        outs = [m["xyz"], m["verts"], m["face_offsets"], m["face_verts"], m["face_tets"], m["face_func"]]
        m.close()
        if it > 0:
            e2e_t.append(time.perf_counter() - t0)
        d2h = sum(o.nbytes for o in outs)
    h2d = sum(f.nbytes for _, f in probs) + 56 * len(probs)
    # the plain drop-in, one call per problem (same descriptors, same results)
    t0 = time.perf_counter()
    plain_dev = 0.0
    for r, f in ([] if args.no_plain else probs):
        m = pkg.grid_implicit_arrangement(r, f)
        plain_dev += m.timings["total"]
        m.close()
    plain_wall = time.perf_counter() - t0
    peak, peak_kind = _peaks()
    stage_ms = {k: statistics.mean(v) for k, v in stage.items()}
    line = {
        "metric": METRIC, "value": value, "unit": "tets/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": wl.name, "tets": wl.n_tets, "verts": wl.n_verts, "problems": len(probs),
                   "functions_per_problem": "2..24", "mode": "ia",
                   "l2": "inputs larger than L2 (padded values %.1f GB)" %
                   (8 * wl.n_verts * max(len(f) for _, f in probs) / 1e9), "parallelism": "single"},
        "stage_ms": stage_ms, "stats": st, "wall_ms_per_step": wall / args.steps * 1e3,
        "e2e": {"value": wl.n_tets / statistics.median(e2e_t) if e2e_t else None, "unit": "tets/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": launches,
        "tuning": tuned if tuned else {"record": pkg.get_tuning()},
        "per_problem_plain": None if args.no_plain else {
            "tets_per_s_wall": wl.n_tets / plain_wall, "wall_s": plain_wall, "device_s": plain_dev,
            "batch_speedup_wall": plain_wall / (wall / args.steps)},
        "roofline": {"bound": "hbm", "kernel_stage": "total", "achieved": None, "peak": peak, "unit": "GB/s",
                     "frac": None, "peak_kind": peak_kind, "traffic": None},
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline:
        rates, _, cores, desc = cpu_batch(probs, "ia")
        line["cpu_baseline"] = {"value": rates[0], "unit": "tets/s", "cores": cores, "kind": "port", "sample": desc}
    print(json.dumps(line))


def run_serve(args, world, local):
    """The served form against the plain drop-in on the same Poisson request stream."""
    import numpy as np
    import torch

    torch.cuda.set_device(local)
    fns = importlib.import_module(PKG + ".functions")
    pkg = importlib.import_module(PKG)
    pkg.build()
    L = pkg.load()
    n = max(1, int(args.rate * args.duration))
    reqs = fns.workload_serve(n=n)
    rng = np.random.default_rng(6)
    gaps = rng.exponential(1.0 / args.rate, size=n)
    arrivals = np.cumsum(gaps) - gaps[0]
    total_tets = sum(r.n_tets for r in reqs)
    # warm-up: every kind once through both paths (tables, caches, pools)
    srv = pkg.Server(budget_bytes=int(args.budget_gb * 2 ** 30), streams=args.streams, max_batch=256)
    for r in reqs[:6]:
        t = srv.submit(r.kind, r.res, r.funcs, tree=r.tree)
        srv.wait(t)
        srv.release(t)
        m = (pkg.grid_material_interface if r.kind == "mi" else pkg.grid_implicit_arrangement)(r.res, r.funcs)
        if r.kind == "csg":
            m.csg(r.tree)
        m.close()
    launches0 = int(L.ria_kernel_launches())
    # served: a submitter replays the arrival times; results are consumed as they complete
    tickets = [None] * n
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()

        def submit():
            for i, r in enumerate(reqs):
                d = t0 + arrivals[i] - time.perf_counter()
                if d > 0:
                    time.sleep(d)
                tickets[i] = srv.submit(r.kind, r.res, r.funcs, tree=r.tree)
        th = threading.Thread(target=submit)
        th.start()
        lat = []
        for i in range(n):
            while tickets[i] is None:
                time.sleep(0.0002)
            _, l = srv.wait(tickets[i])
            lat.append(l)
            srv.release(tickets[i])
        th.join()
        served_wall = time.perf_counter() - t0
    launches = int(L.ria_kernel_launches()) - launches0
    srv.close()
    # plain: one request at a time in arrival order; latency counts the wait in the queue
    plain_lat = []
    t0 = time.perf_counter()
    for i, r in enumerate(reqs):
        d = t0 + arrivals[i] - time.perf_counter()
        if d > 0:
            time.sleep(d)
        m = (pkg.grid_material_interface if r.kind == "mi" else pkg.grid_implicit_arrangement)(r.res, r.funcs)
        if r.kind == "csg":
            m.csg(r.tree)
        m.close()
        plain_lat.append(time.perf_counter() - (t0 + arrivals[i]))
    plain_wall = time.perf_counter() - t0
    pct = lambda v, q: float(np.percentile(np.asarray(v) * 1e3, q))
    peak, peak_kind = _peaks()
    line = {
        "metric": METRIC, "value": total_tets / served_wall, "unit": "tets/s", "n_gpus": world, "steps": 1,
        "warmup": 1, "ms_per_step": served_wall * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": "served-poisson", "requests": n, "rate_per_s": args.rate, "duration_s": args.duration,
                   "mix": "60% ia / 30% mi / 10% csg", "tets": "log-uniform 10k..2M (total %d)" % total_tets,
                   "functions": "2..16", "budget_gb": args.budget_gb, "streams": args.streams,
                   "l2": "inputs generated per request on the device", "parallelism": "single"},
        "latency_ms": {"p50": pct(lat, 50), "p99": pct(lat, 99), "max": pct(lat, 100)},
        "plain": {"p50_ms": pct(plain_lat, 50), "p99_ms": pct(plain_lat, 99), "tets_per_s": total_tets / plain_wall,
                  "wall_s": plain_wall},
        "p99_ratio_plain_over_served": pct(plain_lat, 99) / pct(lat, 99),
        "e2e": {"value": total_tets / served_wall, "unit": "tets/s",
                "h2d_bytes_per_step": int(sum(r.funcs.nbytes for r in reqs)), "d2h_bytes_per_step": 0},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "kernel_stage": "total", "achieved": None, "peak": peak, "unit": "GB/s",
                     "frac": None, "peak_kind": peak_kind, "traffic": None},
        "clocks": clk.summary(),
    }
    print(json.dumps(line))


def algorithmic_bytes(wl, st, n_fit, n_rec, n_face_verts, n_face_tets):
    """Bytes each stage must move at least: n_fit = sum of active functions over the active tets,
    n_rec = record bytes; the extraction reads the active lists and every record once, writes one
    dedup-table slot per distinct vertex key (16 bytes: key and owner), and writes the points, the
    vertex records (11 int64) and the face lists (vertex ids, offsets, (tet, face) pairs, function
    pairs)."""
    V, T, F = wl.n_verts, wl.n_tets, len(wl.funcs)
    A = st["num_intersecting_tet"]
    nv, nf = st["num_verts"], st["num_faces"]
    return {
        "sample": 8 * V * F + 16 * V,           # values written + per-vertex masks written
        "filter": 16 * V + 28 * A,              # masks read once + active-tet lists written
        "cut": 32 * n_fit + n_rec,              # corner values read + records written
        "extract": 20 * A + n_rec + 16 * nv + 24 * nv + 88 * nv + 8 * n_face_verts + 16 * nf + 16 * n_face_tets
                   + 16 * nf,
    }


# FP64 operations per grid vertex of each function kind in the sampler (include/ria.h formulas, with
# the first sum of every formula tabulated per (x, y) column): additions, multiplications
SAMPLE_FP64_OPS = {1: (1, 0), 2: (2, 0), 3: (2, 1), 4: (7, 6), 5: (9, 8), 0: (0, 0)}


def sample_fp64_ops(wl):
    """FP64 additions and multiplications the sampling formulas need over the grid (algorithmic)."""
    per_vertex = sum(sum(SAMPLE_FP64_OPS[int(t)]) for t in wl.funcs["type"])
    return per_vertex * wl.n_verts


# FP64 operations of the vertex coordinates per mesh vertex, by simplex size (the reference's formulas,
# src/extract_mesh.h:111-159; a division counts as one operation): a tet-vertex copies a point, an
# edge vertex 12, a face vertex 29, a vertex inside a tet 84
XYZ_FP64_OPS = {1: 0, 2: 12, 3: 29, 4: 84}

# FP64 pipe busy fraction of the warp cut on this workload, from its ncu capture (heavy bins, light
# bins): the exact predicates run through FP32 and FP64 filters, and few operations reach the pipe
CUT_FP64_PIPE_BUSY = {"kernel": "k_cut_warp", "heavy_bins": 0.111, "light_bins": 0.034,
                      "source": "ncu sm__pipe_fp64_cycles_active, one capture of each launch"}


def fp64_rate(L):
    """Measured FP64 add/mul and fused multiply-add rates of this GPU (ria_measure_fp64_rate)."""
    import ctypes

    out = {}
    for op, name in ((0, "fma"), (1, "add")):
        r = ctypes.c_double()
        out[name] = r.value if L.ria_measure_fp64_rate(op, ctypes.byref(r)) == 0 else None
    return out


def cpu_slabs(wl, parts=3):
    """The workload grid cut into `parts` contiguous x-slabs of cube layers (each re-indexed as a grid
    of its own); together they hold every tet of the grid once."""
    fns = importlib.import_module(PKG + ".functions")
    res = wl.res
    n = res + 1
    pts_all, tets_all = fns.generate_tet_mesh(res, wl.bbox_min, wl.bbox_max)
    per_layer = 5 * res * res
    out = []
    for p in range(parts):
        i0, i1 = res * p // parts, res * (p + 1) // parts
        tets = tets_all[i0 * per_layer:i1 * per_layer] - i0 * n * n
        pts = pts_all[i0 * n * n:(i1 + 1) * n * n]
        out.append((pts, tets, i0, i1))
    return out


def cpu_whole_grid(wl, threads, parts=3):
    """Stages a-d of the CPU restatement over the whole workload grid, in x-slabs: (tets/s over the
    grid, per-slab tets/s, description)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle

    pyoracle.build()
    total_t, total_n, rates = 0.0, 0, []
    for pts, tets, i0, i1 in cpu_slabs(wl, parts):
        t0 = time.perf_counter()
        fv = pyoracle.sample(wl.funcs, pts, threads=threads)
        pyoracle.run(wl.mode, pts, tets, fv, threads=threads)
        dt = time.perf_counter() - t0
        total_t += dt
        total_n += len(tets)
        rates.append(len(tets) / dt)
    desc = (f"the whole grid ({total_n} tets) in {parts} x-slabs of cube layers; stages a-d of the CPU "
            f"restatement (oracle/)")
    return total_n / total_t, rates, desc


def run_reference(args, wl, world):
    """The CPU restatement over the whole workload, every host thread for stages a-c (the extraction is
    serial, as in the reference); each step is one pass over the grid."""
    cores = os.cpu_count() or 1
    vals = []
    for it in range(args.warmup + args.steps):
        v, _, desc = cpu_whole_grid(wl, cores)
        if it >= args.warmup:
            vals.append(v)
    value = statistics.median(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "tets/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": wl.n_tets / value * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": wl.name, "tets": wl.n_tets, "functions": len(wl.funcs), "sample": desc},
        "cpu_baseline": {"value": value, "unit": "tets/s", "cores": cores, "kind": "port",
                         "sample": desc + ", stages a-c on every host thread, extraction single-threaded as in "
                                          "the reference; median of the steps"},
        "e2e": {"value": value, "unit": "tets/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="ia-degenerate", choices=["ia-degenerate", "mi", "ia-small", "batch", "serve"])
    ap.add_argument("--batch-n", type=int, default=4096, help="problems of --config batch")
    ap.add_argument("--rate", type=float, default=100.0, help="--config serve: requests per second")
    ap.add_argument("--duration", type=float, default=10.0, help="--config serve: seconds of arrivals")
    ap.add_argument("--budget-gb", type=float, default=120.0, help="--config serve: HBM budget")
    ap.add_argument("--streams", type=int, default=3, help="--config serve: worker streams")
    ap.add_argument("--res", type=int, default=None, help="grid resolution override (small profiling cases)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer end-to-end leg (profiling runs)")
    ap.add_argument("--no-tune", action="store_true", help="--config batch: keep the current tuning record")
    ap.add_argument("--no-plain", action="store_true", help="--config batch: skip the per-problem plain calls")
    ap.add_argument("--tuning", default=None,
                    help="JSON object of ria_tuning fields set before anything runs, e.g. '{\"heavy_min_k\": 3}'")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.config in ("batch", "serve"):
        if args.impl == "reference":
            if rank == 0 and args.config == "batch":
                run_reference_batch(args, world)
            elif rank == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the served form has no CPU reference "
                                  "arm; run --impl reference on the other configs"}))
        elif rank == 0:
            (run_batch if args.config == "batch" else run_serve)(args, world, local)
        return
    wl = workload(args.config, args.res)

    if args.impl == "reference":
        if rank == 0:
            run_reference(args, wl, world)
        return

    import numpy as np
    import torch

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    pkg = importlib.import_module(PKG)
    pkg.build()
    L = pkg.load()
    if args.tuning:
        pkg.set_tuning(dict(pkg.get_tuning(), **json.loads(args.tuning)))
    grid = pkg.grid_implicit_arrangement if wl.mode == "ia" else pkg.grid_material_interface
    host = pkg.implicit_arrangement if wl.mode == "ia" else pkg.material_interface

    for _ in range(args.warmup):
        m = grid(wl.res, wl.funcs)
        st = m.stats
        m.close()

    # ---- device-resident throughput
    launches0 = int(L.ria_kernel_launches())
    dev_ms, stage = [], {"sample": [], "filter": [], "cut": [], "extract": []}
    with ClockSampler(local) as clk:
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            L.ria_lookup_cache_clear()  # no reuse across steps: each starts from the seeded lookup tables
            m = grid(wl.res, wl.funcs)
            tm = m.timings
            dev_ms.append(tm["total"] * 1e3)
            for k in stage:
                stage[k].append(tm[k] * 1e3)
            m.close()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        wall = time.perf_counter() - t0
    launches = int(L.ria_kernel_launches()) - launches0
    ms = max_over_ranks(statistics.mean(dev_ms), dist, "cuda")
    value = world * wl.n_tets / (ms * 1e-3)

    # ---- end to end through the host-buffer entry points, host buffers in pinned memory
    fns = importlib.import_module(PKG + ".functions")
    pts, tets = fns.generate_tet_mesh(wl.res, wl.bbox_min, wl.bbox_max)

    def pinned(shape, dtype):
        t = torch.empty(int(np.prod(shape)) * np.dtype(dtype).itemsize, dtype=torch.uint8, pin_memory=True)
        return t.numpy().view(dtype).reshape(shape)

    pts_h = pinned(pts.shape, np.float64)
    pts_h[...] = pts
    tets_h = pinned(tets.shape, np.int64)
    tets_h[...] = tets
    fv_h = pinned((len(pts), len(wl.funcs)), np.float64)
    out_bufs = {}
    names = ["xyz", "verts", "face_offsets", "face_verts", "face_tets", "face_func"]
    e2e_times = []
    h2d = d2h = 0
    for it in range(0 if args.no_e2e else 1 + args.steps):
        L.ria_lookup_cache_clear()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fv = pkg.sample_functions(wl.funcs, pts_h, out=fv_h)
        m = host(pts_h, tets_h, fv)
        if it == 0:  # size the pinned result buffers once (untimed iteration)
            for k in names:
                n = int(L.ria_mesh_count(m._h, pkg.Mesh._FIELDS[k][0]))
                out_bufs[k] = pinned((max(n, 1) * 2,), pkg.Mesh._FIELDS[k][1])
        outs = [m.copy_into(k, out_bufs[k]) for k in names]
        m.close()
        dt = time.perf_counter() - t0
        if it > 0:
            e2e_times.append(dt)
        h2d = pts_h.nbytes + wl.funcs.nbytes + pts_h.nbytes + tets_h.nbytes + fv.nbytes
        d2h = fv.nbytes + sum(o.nbytes for o in outs)
    e2e = world * wl.n_tets / max_over_ranks(statistics.median(e2e_times), dist, "cuda") if e2e_times else None

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    peak, peak_kind = _peaks()
    m = grid(wl.res, wl.funcs)  # counts for the byte model (untimed)
    n_fit, n_rec = len(m["func_in_tet"]), len(m["rec_bytes"])
    n_fvert = int(L.ria_mesh_count(m._h, pkg.Mesh._FIELDS["face_verts"][0]))
    n_ftet = int(L.ria_mesh_count(m._h, pkg.Mesh._FIELDS["face_tets"][0])) // 2
    simplex = np.bincount(m["verts"][:, 2], minlength=5) if wl.mode == "ia" else None
    m.close()
    ab = algorithmic_bytes(wl, st, n_fit, n_rec, n_fvert, n_ftet)
    stage_ms = {k: statistics.mean(v) for k, v in stage.items()}
    rates = fp64_rate(L)
    # the dominant kernel is the sampler (the largest share of the launch list); it is bound by the
    # FP64 pipe, so its FP64 fraction is reported beside its HBM fraction
    dom = "sample"
    achieved = ab[dom] / (stage_ms[dom] * 1e-3) / 1e9
    ops = sample_fp64_ops(wl) if wl.mode in ("ia", "mi") else None
    fp64 = {"kernel": "k_sample", "ops_per_launch": ops,
            "achieved": ops / (stage_ms[dom] * 1e-3) / 1e9 if ops else None,
            "peak": rates["add"] / 1e9 if rates.get("add") else None, "unit": "G FP64 add/mul per s",
            "peak_kind": "measured (ria_measure_fp64_rate, this run)"}
    fp64["frac"] = fp64["achieved"] / fp64["peak"] if fp64["achieved"] and fp64["peak"] else None
    # every stage's FP64 fraction beside its HBM one: the sampler's formulas, none in the IA filter
    # (sign masks only), the cut's from its ncu capture, the vertex coordinates' formulas
    xyz_ops = int(sum(XYZ_FP64_OPS[t] * int(simplex[t]) for t in XYZ_FP64_OPS)) if simplex is not None else None
    peak_ops = fp64["peak"] * 1e9 if fp64["peak"] else None
    stage_fp64 = {
        "sample": fp64["frac"],
        "filter": 0.0 if wl.mode == "ia" else None,
        "cut": CUT_FP64_PIPE_BUSY if wl.name == SAMPLE_TRAFFIC_WORKLOAD else None,
        "extract": xyz_ops / (stage_ms["extract"] * 1e-3) / peak_ops if xyz_ops is not None and peak_ops else None,
    }
    line = {
        "metric": METRIC, "value": value, "unit": "tets/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": wl.name, "tets": wl.n_tets, "verts": wl.n_verts, "functions": len(wl.funcs),
                   "mode": wl.mode, "l2": "inputs larger than L2 (V x F FP64 values %.0f MB)" %
                   (8 * wl.n_verts * len(wl.funcs) / 1e6), "parallelism": "replicas" if world > 1 else "single"},
        "stage_ms": stage_ms,
        "stats": st,
        "wall_ms_per_step": wall / args.steps * 1e3,
        "e2e": {"value": e2e, "unit": "tets/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": launches,
        "tuning": pkg.get_tuning(),
        "roofline": {"bound": "hbm", "kernel": "k_sample", "kernel_stage": dom, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                     "algorithmic_bytes": ab[dom], "traffic": SAMPLE_TRAFFIC if wl.name == SAMPLE_TRAFFIC_WORKLOAD else None,
                     "fp64": fp64,
                     "stage_frac": {k: ab[k] / (stage_ms[k] * 1e-3) / 1e9 / peak for k in stage_ms},
                     "stage_fp64_frac": stage_fp64,
                     "stage_algorithmic_bytes": ab,
                     "note": "sampling is bound by the FP64 pipe (fp64.frac); the cut and the extraction are "
                             "latency-bound (see the ncu summaries): their HBM fractions are low"},
        "clocks": clk.summary(),
    }
    if not args.no_cpu_baseline:
        runs = [cpu_whole_grid(wl, 1) for _ in range(3)]
        v = statistics.median(r[0] for r in runs)
        per_slab, desc = runs[0][1], runs[0][2]
        line["cpu_baseline"] = {"value": v, "unit": "tets/s", "cores": 1, "kind": "port",
                                "sample": desc + ", one thread, median of 3 passes (" +
                                          ", ".join("%.3g" % r[0] for r in runs) + " tets/s); tets/s per slab "
                                          "in the first pass " + ", ".join("%.3g" % r for r in per_slab)}
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
