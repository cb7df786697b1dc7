#!/usr/bin/env python3
"""Benchmark of the GB300 capacitance solve path.

Metric: solves/s of one complete capacitance extraction (GPU coefficient fill
+ batched preconditioned GMRES + capacitance assembly) of a resident model,
with p50/p99 step latency, for the mixed-precision path (headline) beside the
plain FP64 path, and the end-to-end figure through the C ABI with the model
uploaded from pinned host memory and the capacitance matrix read back.

Workload (default): single conductor sphere, radius 1 m, icosahedron
subdivided 7 times (327,680 triangles), mesh refinement off (-m1e30), link
tolerance 3e-4 (-d3e-34), GMRES tolerance 1e-4, Jacobi preconditioner.
Synthetic, generated deterministically by fastercap_gb300.geometry.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

N > 1 runs replicas (one independent workload per GPU, launched by torchrun).
--impl reference times the reference algorithm's CPU implementation (the
oracle port; the reference's own binary where it was built on this machine)
on all host cores, on the same model.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FOUR_PI_E0 = 1.1126500559756e-10
METRIC = "solves/s & p50/p99 latency, mixed vs FP64 on GB300 at <=0.1% C-matrix error"

WORKLOADS = {
    # name: (writer, mesh_eps, eps_ratio, gmres tol, analytic C or None)
    "sphere_327680": (lambda p: __import__("fastercap_gb300.geometry", fromlist=["x"]).write_sphere(p, 7),
                      1e30, 3e-34, 1e-4, FOUR_PI_E0),
    "sphere_81920": (lambda p: __import__("fastercap_gb300.geometry", fromlist=["x"]).write_sphere(p, 6),
                     1e30, 1e-33, 1e-4, FOUR_PI_E0),
    "sphere_20480": (lambda p: __import__("fastercap_gb300.geometry", fromlist=["x"]).write_sphere(p, 5),
                     1e30, 1e-33, 1e-4, FOUR_PI_E0),
    # 8x8 bus crossing (16 conductors) in an eps_r=3.9 slab under a planar
    # interface to eps_r=1: 130,942 panels, 81.4M links, 16 right-hand sides
    "crossing8x8_slab": (lambda p: __import__("fastercap_gb300.geometry", fromlist=["x"]).crossing_8x8_slab().write(p),
                         5e-6, 1.0, 1e-4, None),
}

# many independent geometries in one problem: name -> (crossing list,
# mesh_eps, eps_ratio, gmres tol). crossings32: 32 random k x k crossings in
# vacuum drawn in order from default_rng(0) (k in 2..10, length 10-60 um,
# pitch 2-4 um, gap 1-3 um): 4,736 to 48,128 panels each, 765,504 panels,
# 428 conductors and 255.2M links in all.
MULTI = {
    "crossings32": (lambda: __import__("fastercap_gb300.geometry", fromlist=["x"]).crossing_batch(0, 32, 2, 10),
                    1e-3, 1.0, 1e-4),
}


# DRAM bytes per link-product launch (dram__bytes_read.sum +
# dram__bytes_write.sum) from one ncu capture of the same kernel and workload
LINK_TRAFFIC = {
    "sphere_327680": 534.116864e6 + 4.707072e6,    # k_spmv32<1, 16>
    "crossing8x8_slab": 679.950848e6 + 7.460608e6,  # k_spmv32_multi<16>
}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    from fastercap_gb300 import replicas
    return replicas.dist_env()


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    PERIOD_S = 0.05

    def __init__(self, device: int):
        self.device = device
        self.samples = []  # (host time, fields)
        self.proc = None
        self.t_start = self.t_end = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", str(int(self.PERIOD_S * 1000))],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            # the timed region starts once the sampler is live (at most 3 s)
            t0 = time.perf_counter()
            while not self.samples and self.proc.poll() is None and time.perf_counter() - t0 < 3.0:
                time.sleep(0.005)
        except (OSError, FileNotFoundError):
            self.proc = None
        self.t_start = time.perf_counter()
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.samples.append((time.perf_counter(), parts))

    def __exit__(self, *a):
        self.t_end = time.perf_counter()
        if self.proc:
            time.sleep(self.PERIOD_S * 1.5)  # the sample in flight at the end of the region
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        """Samples taken inside the timed region and the first one after its
        end (a region shorter than the sampling period still gets one)."""
        inside = [p for t, p in self.samples if self.t_start <= t <= self.t_end]
        after = [p for t, p in self.samples if self.t_end is not None and t > self.t_end]
        use = inside + after[:1]
        if not use:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(s[0]) for s in use if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in use if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in use for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(use), "period_ms": int(self.PERIOD_S * 1000)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def build_multi(workload: str, ctx=None):
    """(concatenated model, geometry_of_conductor, [per-geometry models], build s, tol, link eps);
    with a context the link construction of every geometry runs on its GPU"""
    import fastercap_gb300 as fc
    make, meps, dratio, tol = MULTI[workload]
    models = []
    t0 = time.perf_counter()
    with tempfile.TemporaryDirectory() as tmp:
        for g, cr in enumerate(make()):
            path = os.path.join(tmp, "g%d.txt" % g)
            cr.write(path)
            models.append(fc.Model.build(path, mesh_eps=meps, eps_ratio=dratio, ctx=ctx))
    model, geom = fc.Model.concat(models)
    return model, geom, models, time.perf_counter() - t0, tol, meps * dratio


def build_model(workload: str, ctx=None, compare=False):
    """(model, build s, tol, analytic C, link eps). With a context the link
    construction runs on its GPU; `compare` also builds on the host alone and
    returns its time as a sixth value after checking that the models agree."""
    import fastercap_gb300 as fc
    writer, meps, dratio, tol, analytic = WORKLOADS[workload]
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, workload + ".txt")
        writer(path)
        t0 = time.perf_counter()
        model = fc.Model.build(path, mesh_eps=meps, eps_ratio=dratio, ctx=ctx)
        build_s = time.perf_counter() - t0
        if not compare:
            return model, build_s, tol, analytic, meps * dratio
        t0 = time.perf_counter()
        host = fc.Model.build(path, mesh_eps=meps, eps_ratio=dratio)
        host_s = time.perf_counter() - t0
    for k in ("link_ptr", "link_src", "node_left", "node_vertices"):
        if not np.array_equal(model.arrays[k], host.arrays[k]):
            raise RuntimeError("device-built model differs from the host build in " + k)
    del host
    return model, build_s, tol, analytic, meps * dratio, host_s


def model_bytes(model) -> int:
    return int(sum(np.asarray(v).nbytes for v in model.arrays.values()))


def pinned_model(model):
    """Copy the model arrays into pinned host memory (the e2e upload source)."""
    import torch
    import fastercap_gb300 as fc
    arrays, keep = {}, []
    for k, v in model.arrays.items():
        a = np.ascontiguousarray(v)
        t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True)
        view = t.numpy().view(a.dtype).reshape(a.shape)
        view[...] = a
        arrays[k] = view
        keep.append(t)
    m = fc.Model.from_arrays(arrays, list(model.names))
    m._pinned = keep
    return m


def run_reference(args, rank, world):
    """CPU arm: the oracle port on every host core, full solves of the same model."""
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from pyoracle import Oracle
    from fastercap_gb300 import build as fbuild
    fbuild.build(reference=False)
    model, build_s, tol, analytic, eps = build_model(args.workload)
    cores = os.cpu_count() or 1
    o = Oracle(model.arrays, threads=cores)
    times = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        o.fill()
        cap, it, _, _ = o.solve(tol, 1)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(dt)
    total = sum(times)
    value = len(times) / total
    sample = "full solves (fill + GMRES + C) of the %d-panel, %d-link model" % (model.n_panels, model.n_links)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "p50_ms": 1000 * float(np.percentile(times, 50)), "p99_ms": 1000 * float(np.percentile(times, 99)),
        "config": {"workload": args.workload, "panels": model.n_panels, "links": model.n_links, "link_eps": eps,
                   "gmres_tol": tol, "precond": "jacobi", "rhs": len(model.conductor_names)},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "capacitance": float(cap[0, 0]), "iterations": [int(x) for x in it],
    }
    print(json.dumps(line), flush=True)


def run_reference_multi(args, rank, world):
    """CPU arm for a multi-geometry workload: the oracle port on every host
    core; each step solves one geometry (cycling through them in order)."""
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from pyoracle import Oracle
    from fastercap_gb300 import build as fbuild
    fbuild.build(reference=False)
    model, geom, models, build_s, tol, eps = build_multi(args.workload)
    cores = os.cpu_count() or 1
    times, panels = [], []
    for i in range(args.warmup + args.steps):
        m = models[i % len(models)]
        o = Oracle(m.arrays, threads=cores)
        t0 = time.perf_counter()
        o.fill()
        o.solve(tol, 1)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(dt)
            panels.append(m.n_panels)
    total = sum(times)
    value = len(times) / total
    sample = ("one geometry per step, cycling through the %d in order (steps %d..%d: %d panels in all)"
              % (len(models), args.warmup, args.warmup + args.steps - 1, sum(panels)))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "p50_ms": 1000 * float(np.percentile(times, 50)), "p99_ms": 1000 * float(np.percentile(times, 99)),
        "config": {"workload": args.workload, "geometries": len(models), "panels": model.n_panels,
                   "links": model.n_links, "link_eps": eps, "gmres_tol": tol, "precond": "jacobi",
                   "solve": "one geometry's full capacitance matrix (fill + GMRES per conductor + C)"},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def time_steps_multi(prob, stream, n, tol, flush_buf, torch, geom=None, rhs_width=0):
    s = torch.cuda.ExternalStream(stream)
    times, caps, its = [], None, None
    for _ in range(n):
        with torch.cuda.stream(s):
            flush_buf.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        prob.fill()
        caps, its = prob.solve(tol=tol, rhs_width=rhs_width)
        e1.record(s)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    return times, caps, its


def run_gb300_multi(args, rank, world, local_rank):
    """All geometries in one problem: every kernel launch covers all of them,
    each geometry keeps its own GMRES solves."""
    import torch
    import fastercap_gb300 as fc
    from fastercap_gb300 import build as fbuild
    fbuild.build(reference=False)
    torch.cuda.set_device(local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    ctx = fc.Context(local_rank)
    model, geom, models, build_s, tol, eps = build_multi(args.workload, ctx)
    G = len(models)
    stream = ctx.stream
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    prob = ctx.problem(model, fc.PREC_MIXED)
    prob.set_geometries(geom)
    time_steps_multi(prob, stream, args.warmup, tol, flush, torch)
    prob.reset_stats()
    barrier()
    with ClockSampler(local_rank) as clk:
        times, caps_m, its_m = time_steps_multi(prob, stream, args.steps, tol, flush, torch)
    barrier()
    st_timed = prob.stats()
    # link-product roofline: the same steps again with CUDA events around
    # every link-product launch (the timed steps run each Arnoldi loop as one
    # CUDA graph, which cannot bracket single kernels)
    prob.reset_stats()
    prob.set_profiling(True)
    time_steps_multi(prob, stream, max(1, min(args.steps, 3)), tol, flush, torch)
    st = prob.stats()
    prob.set_profiling(False)
    total_ms = sum(times)
    # FP64, same batching
    p64 = ctx.problem(model, fc.PREC_FP64)
    p64.set_geometries(geom)
    time_steps_multi(p64, stream, 1, tol, flush, torch)
    times64, caps_64, its_64 = time_steps_multi(p64, stream, max(1, min(args.steps, 3)), tol, flush, torch)
    p64.close()
    # plain FP64 single right-hand side: one problem per geometry, one
    # conductor at a time
    singles = []
    for m in models:
        q = ctx.problem(m, fc.PREC_FP64)
        singles.append(q)
    for q in singles:
        q.fill()
        q.solve(tol=tol, rhs_width=1)
    torch.cuda.synchronize()
    s = torch.cuda.ExternalStream(stream)
    with torch.cuda.stream(s):
        flush.zero_()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for q in singles:
        q.fill()
        q.solve(tol=tol, rhs_width=1)
    e1.record(s)
    e1.synchronize()
    single_ms = e0.elapsed_time(e1)
    for q in singles:
        q.close()
    # end to end through the C ABI: pinned host model -> upload -> fill -> solve -> C back
    pm = pinned_model(model)
    h2d = model_bytes(model)
    e2e_times = []
    for i in range(args.warmup + args.steps):
        with torch.cuda.stream(s):
            flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        pe = ctx.problem(pm, fc.PREC_MIXED)
        pe.set_geometries(geom)
        pe.fill()
        caps_e, its_e = pe.solve(tol=tol)
        e1.record(s)
        e1.synchronize()
        pe.close()
        if i >= args.warmup:
            e2e_times.append(e0.elapsed_time(e1))
    d2h = sum(c.nbytes for c in caps_e) + 4 * sum(len(i) for i in its_e)
    from fastercap_gb300 import replicas
    tmax, e2e_max = replicas.max_over_ranks([total_ms, sum(e2e_times)], world)
    value = replicas.throughput(args.steps * G, world, tmax / 1000.0)
    e2e_value = replicas.throughput(args.steps * G, world, e2e_max / 1000.0)
    peak, peak_kind = peaks()
    link_avg_ms = st["link_ms"] / max(1, st["link_launches"])
    link_bytes = st["link_bytes"] / max(1, st["link_launches"])
    achieved = link_bytes / (link_avg_ms / 1000.0) / 1e9 if link_avg_ms > 0 else None
    err_m64 = max(float(np.max(np.abs(a - b) / np.abs(b))) for a, b in zip(caps_m, caps_64))
    it_all = np.concatenate([np.asarray(i) for i in its_m])
    result = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 links / f64 Krylov", "data": "synthetic",
        "p50_ms": float(np.percentile(times, 50)), "p99_ms": float(np.percentile(times, 99)),
        "config": {"workload": args.workload, "geometries": G, "panels": model.n_panels, "links": model.n_links,
                   "panels_min_max": [min(m.n_panels for m in models), max(m.n_panels for m in models)],
                   "link_eps": eps, "gmres_tol": tol, "precond": "jacobi",
                   "rhs": int(sum(len(m.conductor_names) for m in models)),
                   "solve": "one geometry's full capacitance matrix; a step solves all geometries in one problem",
                   "l2": "flushed between steps (256 MiB write); links exceed L2", "host_build_s": round(build_s, 3),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "fp64": {"value": world * len(times64) * G / (sum(times64) / 1000.0), "unit": "solves/s",
                 "p50_ms": float(np.percentile(times64, 50))},
        "fp64_single_rhs": {"value": G / (single_ms / 1000.0), "unit": "solves/s", "ms_all_geometries": single_ms,
                            "note": "one FP64 problem per geometry, one right-hand side at a time"},
        "mixed_vs_fp64": {"speedup": (sum(times64) / len(times64)) / (total_ms / args.steps),
                          "speedup_vs_single_rhs": single_ms / (total_ms / args.steps), "max_rel_c_err": err_m64},
        "accuracy": {"iterations_min_max": [int(it_all.min()), int(it_all.max())]},
        "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "p50_ms": float(np.percentile(e2e_times, 50))},
        "gpu_launches": int(st_timed["kernel_launches"]),
        "phases": {"fill_ms_last": st_timed["fill_ms"], "solve_ms_last": st_timed["solve_ms"],
                   "fill_fp64_coefficients": st_timed["fill_fp64"]},
        "roofline": {"kernel": "link product (k_spmv32_multi)", "bound": "hbm",
                     "timing": "CUDA events around every link-product launch, steps re-run after the timed region",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "peak_source": peak_kind,
                     "traffic": None, "launches": int(st["link_launches"]),
                     "bytes_per_launch": link_bytes, "avg_launch_ms": link_avg_ms},
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        from pyoracle import Oracle
        cores = os.cpu_count() or 1
        t0 = time.perf_counter()
        n_done, errs = 0, []
        for m, cm in zip(models, caps_m):
            o = Oracle(m.arrays, threads=cores)
            o.fill()
            ocap, _, _, _ = o.solve(tol, 1)
            errs.append(float(np.max(np.abs(cm - ocap) / np.abs(ocap))))
            n_done += 1
            if time.perf_counter() - t0 > 20.0:
                break
        dt = time.perf_counter() - t0
        result["cpu_baseline"] = {"value": n_done / dt, "unit": "solves/s", "cores": cores, "kind": "port",
                                  "sample": "the first %d geometries in order, one full solve each" % n_done}
        result["accuracy"]["max_rel_c_err_vs_cpu_fp64"] = max(errs)
    if rank == 0:
        print(json.dumps(result), flush=True)
    prob.close()
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


# Serving: request r is random_crossing(r) with k in 2..12 (numpy
# default_rng(r)); arrivals are Poisson at rate lam with inter-arrival times
# from default_rng(10000 + lam). Host models are built before the clock
# starts (the solve is measured from an uploaded host model).
SERVING = {"mesh_eps": 1e-3, "tol": 1e-4, "kmin": 2, "kmax": 12}


def build_requests(n: int, rank: int = 0, world: int = 1):
    import fastercap_gb300 as fc
    from fastercap_gb300 import geometry as geo
    from concurrent.futures import ThreadPoolExecutor
    tmp = tempfile.mkdtemp()

    def one(r):
        path = os.path.join(tmp, "req%d.txt" % r)
        geo.random_crossing(r, SERVING["kmin"], SERVING["kmax"]).write(path)
        m = fc.Model.build(path, mesh_eps=SERVING["mesh_eps"])
        os.unlink(path)
        return m

    from fastercap_gb300 import replicas
    ids = replicas.shard(n, rank, world)  # request r is served by GPU r mod world
    t0 = time.perf_counter()
    with ThreadPoolExecutor(os.cpu_count() or 1) as ex:  # the native builder releases the GIL
        models = list(ex.map(one, ids))
    os.rmdir(tmp)
    return models, ids, time.perf_counter() - t0


def serve_pass(srv, models, ids, n_total, precision, lam, tol, world=1):
    """Submit every request of this GPU's shard at its arrival time (one
    Poisson schedule over all n_total requests); returns per-request
    (latency ms, completion s, C, iterations, info)."""
    arr = np.cumsum(np.random.default_rng(10000 + int(lam)).exponential(1.0 / lam, n_total))
    from fastercap_gb300 import replicas
    replicas.barrier(world)
    t0 = time.perf_counter()
    sub = []
    for r, m in zip(ids, models):
        dt = t0 + arr[r] - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        ts = time.perf_counter()
        sub.append((ts, srv.submit(m, precision, tol=tol)))
    out = []
    for ts, j in sub:
        cap, it = j.result()
        lat = j.info["queue_ms"] + j.info["run_ms"]
        out.append((lat, ts - t0 + lat / 1000.0, cap, it, j.info))
    return out


def run_serving(args, rank, world, local_rank):
    import torch
    import fastercap_gb300 as fc
    from fastercap_gb300 import build as fbuild
    fbuild.build(reference=False)
    torch.cuda.set_device(local_rank)
    from fastercap_gb300 import replicas
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    rates = [float(x) for x in args.rates.split(",")]
    models, ids, build_s = build_requests(args.requests, rank, world)
    ctx = fc.Context(local_rank)
    tol = SERVING["tol"]
    res = {}
    caps = {}
    launches = 0
    clk_summary = None
    with ctx.server(slots=args.slots) as srv:
        # warm the pool and the kernels
        for j in [srv.submit(m, fc.PREC_MIXED, tol=tol) for m in models[:4]]:
            j.result()
        for prec, name in ((fc.PREC_MIXED, "mixed"), (fc.PREC_FP64, "fp64")):
            res[name] = {}
            for lam in rates:
                if name == "mixed" and lam == rates[-1]:
                    with ClockSampler(local_rank) as clk:
                        out = serve_pass(srv, models, ids, args.requests, prec, lam, tol, world)
                    clk_summary = clk.summary()
                else:
                    out = serve_pass(srv, models, ids, args.requests, prec, lam, tol, world)
                # latencies of every GPU's shard; the job ends with the slowest GPU
                parts = replicas.gather_to_all(([o[0] for o in out], max(o[1] for o in out)), world)
                lat = np.array([x for p_ in parts for x in p_[0]])
                span = max(p_[1] for p_ in parts)
                res[name][str(int(lam))] = {"solves_s": len(lat) / span, "p50_ms": float(np.percentile(lat, 50)),
                                            "p99_ms": float(np.percentile(lat, 99)),
                                            "mean_queue_ms": float(np.mean([o[4]["queue_ms"] for o in out]))}
                caps[(name, lam)] = [o[2] for o in out]
                if name == "mixed" and lam == rates[-1]:
                    launches = int(sum(o[4]["kernel_launches"] for o in out))
        st = srv.stats()
    top = str(int(rates[-1]))
    err = max(float(np.max(np.abs(a - b) / np.abs(b))) for a, b in zip(caps[("mixed", rates[-1])], caps[("fp64", rates[-1])]))
    # the same request gives the same matrix at every rate (alone or in any mix)
    same = all(np.array_equal(a, b) for lam in rates for a, b in zip(caps[("mixed", lam)], caps[("mixed", rates[0])]))
    h2d = int(np.mean([model_bytes(m) for m in models]))
    mixed_top = res["mixed"][top]
    result = {
        "metric": METRIC, "value": mixed_top["solves_s"], "unit": "solves/s", "n_gpus": world, "steps": args.requests,
        "warmup": 4, "ms_per_step": 1000.0 / mixed_top["solves_s"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 links / f64 Krylov", "data": "synthetic",
        "p50_ms": mixed_top["p50_ms"], "p99_ms": mixed_top["p99_ms"],
        "config": {"workload": "serving", "requests": args.requests, "rates_req_s": rates, "slots": args.slots,
                   "parallelism": "request r on GPU r mod N" if world > 1 else "single GPU",
                   "request": "random k x k crossing, k in 2..12, seed = request id", "link_eps": SERVING["mesh_eps"],
                   "gmres_tol": tol, "precond": "jacobi",
                   "panels_min_max_mean": [min(m.n_panels for m in models), max(m.n_panels for m in models),
                                           int(np.mean([m.n_panels for m in models]))],
                   "links_mean": int(np.mean([m.n_links for m in models])), "host_build_s": round(build_s, 2),
                   "step": "one request (upload + fill + GMRES + C), value at the highest rate",
                   "l2": "each request's links exceed L2 on average; no flush"},
        "serving": res,
        "mixed_vs_fp64": {"speedup_at_top_rate": mixed_top["solves_s"] / res["fp64"][top]["solves_s"],
                          "max_rel_c_err": err},
        "same_result_every_rate": bool(same),
        "server": {"max_running": st["max_running"], "peak_in_use_bytes": st["peak_in_use"], "budget_bytes": st["budget"]},
        "e2e": {"value": mixed_top["solves_s"], "unit": "solves/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": int(np.mean([c.nbytes for c in caps[("mixed", rates[-1])]]))},
        "gpu_launches": launches,
        "clocks": clk_summary,
    }
    if not args.no_cpu_baseline and rank == 0 and world == 1:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        from pyoracle import Oracle
        cores = os.cpu_count() or 1
        t0 = time.perf_counter()
        n = 0
        for m in models:
            o = Oracle(m.arrays, threads=cores)
            o.fill()
            o.solve(tol, 1)
            n += 1
            if time.perf_counter() - t0 > 20.0:
                break
        dt = time.perf_counter() - t0
        result["cpu_baseline"] = {"value": n / dt, "unit": "solves/s", "cores": cores, "kind": "port",
                                  "sample": "the first %d requests, solved one after another" % n}
    if rank == 0:
        print(json.dumps(result), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def run_reference_serving(args, rank, world):
    """CPU arm for serving: the oracle port on every host core solves the
    requests one after another (the first steps + warmup requests)."""
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from pyoracle import Oracle
    from fastercap_gb300 import build as fbuild
    fbuild.build(reference=False)
    models, _, build_s = build_requests(args.warmup + args.steps)
    cores = os.cpu_count() or 1
    times = []
    for i, m in enumerate(models):
        o = Oracle(m.arrays, threads=cores)
        t0 = time.perf_counter()
        o.fill()
        o.solve(SERVING["tol"], 1)
        if i >= args.warmup:
            times.append(time.perf_counter() - t0)
    total = sum(times)
    value = len(times) / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "p50_ms": 1000 * float(np.percentile(times, 50)), "p99_ms": 1000 * float(np.percentile(times, 99)),
        "config": {"workload": "serving", "requests": args.steps, "link_eps": SERVING["mesh_eps"],
                   "gmres_tol": SERVING["tol"], "precond": "jacobi"},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port",
                         "sample": "requests %d..%d solved one after another (no arrival process)"
                                   % (args.warmup, args.warmup + args.steps - 1)},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def time_steps(prob, stream, n, tol, flush_buf, torch):
    """Per-step device times (ms) of fill + solve, L2 flushed between steps."""
    s = torch.cuda.ExternalStream(stream)
    times, cap, it = [], None, None
    for _ in range(n):
        with torch.cuda.stream(s):
            flush_buf.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        prob.fill()
        cap, it = prob.solve(tol=tol)
        e1.record(s)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    return times, cap, it


def run_gb300(args, rank, world, local_rank):
    import torch
    import fastercap_gb300 as fc
    from fastercap_gb300 import build as fbuild
    fbuild.build(reference=False)
    torch.cuda.set_device(local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    ctx = fc.Context(local_rank)
    compare = rank == 0 and world == 1
    built = build_model(args.workload, ctx, compare=compare)
    model, build_s, tol, analytic, eps = built[:5]
    host_build_s = built[5] if compare else None
    stream = ctx.stream
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # resident mixed-precision problem: the headline
    prob = ctx.problem(model, fc.PREC_MIXED)
    time_steps(prob, stream, args.warmup, tol, flush, torch)
    prob.reset_stats()
    barrier()
    with ClockSampler(local_rank) as clk:
        times, cap_m, it_m = time_steps(prob, stream, args.steps, tol, flush, torch)
    barrier()
    st_timed = prob.stats()
    phase = {"fill_ms_last": st_timed["fill_ms"], "solve_ms_last": st_timed["solve_ms"],
             "fill_fp64_coefficients": st_timed["fill_fp64"]}
    # link-product roofline: the same steps again with CUDA events around
    # every link-product launch (the timed steps run each Arnoldi loop as one
    # CUDA graph, which cannot bracket single kernels)
    prob.reset_stats()
    prob.set_profiling(True)
    time_steps(prob, stream, args.steps, tol, flush, torch)
    st = prob.stats()
    prob.set_profiling(False)
    total_ms = sum(times)
    # plain FP64 path on the same model
    p64 = ctx.problem(model, fc.PREC_FP64)
    time_steps(p64, stream, max(1, args.warmup), tol, flush, torch)
    times64, cap_64, it_64 = time_steps(p64, stream, args.steps, tol, flush, torch)
    p64.close()
    # end to end through the C ABI: pinned host model -> upload -> fill -> solve -> C back
    pm = pinned_model(model)
    h2d = model_bytes(model)
    s = torch.cuda.ExternalStream(stream)
    e2e_times = []
    for i in range(args.warmup + args.steps):
        with torch.cuda.stream(s):
            flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        pe = ctx.problem(pm, fc.PREC_MIXED)
        pe.fill()
        cap_e, _ = pe.solve(tol=tol)
        e1.record(s)
        e1.synchronize()
        pe.close()
        if i >= args.warmup:
            e2e_times.append(e0.elapsed_time(e1))
    d2h = cap_e.nbytes + 4 * len(cap_e)

    from fastercap_gb300 import replicas
    tmax, e2e_max = replicas.max_over_ranks([total_ms, sum(e2e_times)], world)
    value = replicas.throughput(args.steps, world, tmax / 1000.0)
    e2e_value = replicas.throughput(args.steps, world, e2e_max / 1000.0)
    peak, peak_kind = peaks()
    link_avg_ms = st["link_ms"] / max(1, st["link_launches"])
    link_bytes = st["link_bytes"] / max(1, st["link_launches"])
    achieved = link_bytes / (link_avg_ms / 1000.0) / 1e9 if link_avg_ms > 0 else None
    rel_mixed_vs_64 = float(np.max(np.abs(cap_m - cap_64) / np.abs(cap_64)))
    result = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 links / f64 Krylov", "data": "synthetic",
        "p50_ms": float(np.percentile(times, 50)), "p99_ms": float(np.percentile(times, 99)),
        "config": {"workload": args.workload, "panels": model.n_panels, "links": model.n_links, "link_eps": eps,
                   "gmres_tol": tol, "precond": "jacobi", "rhs": len(model.conductor_names),
                   "l2": "flushed between steps (256 MiB write)",
                   "model_build_s": {"gpu_links": round(build_s, 3),
                                     "host": round(host_build_s, 3) if host_build_s is not None else None},
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "fp64": {"value": world * args.steps / (sum(times64) / 1000.0), "unit": "solves/s",
                 "p50_ms": float(np.percentile(times64, 50)), "p99_ms": float(np.percentile(times64, 99)),
                 "iterations": [int(x) for x in it_64]},
        "mixed_vs_fp64": {"speedup": (sum(times64) / sum(times)), "max_rel_c_err": rel_mixed_vs_64},
        "accuracy": {"c_mixed": float(cap_m[0, 0]), "c_fp64": float(cap_64[0, 0]),
                     "rel_err_vs_analytic": (float(cap_m[0, 0]) - analytic) / analytic if analytic else None,
                     "min_abs_c_over_diag": float(np.min(np.abs(cap_64) / np.abs(np.diag(cap_64))[:, None])),
                     "iterations": [int(x) for x in it_m]},
        "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "p50_ms": float(np.percentile(e2e_times, 50))},
        "gpu_launches": int(st_timed["kernel_launches"]),
        "phases": phase,
        "roofline": {"kernel": "k_spmv32<1, lanes> (link product)" if len(model.conductor_names) == 1
                     else "k_spmv32_multi (link product)", "bound": "hbm",
                     "timing": "CUDA events around every link-product launch, same steps re-run after the timed region",
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "peak_source": peak_kind,
                     "traffic": LINK_TRAFFIC.get(args.workload), "launches": int(st["link_launches"]),
                     "bytes_per_launch": link_bytes, "avg_launch_ms": link_avg_ms},
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        from pyoracle import Oracle
        cores = os.cpu_count() or 1
        o = Oracle(model.arrays, threads=cores)
        t0 = time.perf_counter()
        o.fill()
        ocap, oit, _, _ = o.solve(tol, 1)
        dt = time.perf_counter() - t0
        result["cpu_baseline"] = {"value": 1.0 / dt, "unit": "solves/s", "cores": cores, "kind": "port",
                                  "sample": "one full solve (fill + GMRES + C) of the same model"}
        result["accuracy"]["max_rel_c_err_vs_cpu_fp64"] = float(np.max(np.abs(cap_m - ocap) / np.abs(ocap)))
    if rank == 0:
        print(json.dumps(result), flush=True)
    prob.close()
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="sphere_327680", choices=sorted(WORKLOADS) + sorted(MULTI) + ["serving"])
    ap.add_argument("--requests", type=int, default=200, help="serving: number of requests")
    ap.add_argument("--rates", default="50,200,500", help="serving: arrival rates (req/s), comma separated")
    ap.add_argument("--slots", type=int, default=4, help="serving: concurrent jobs")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        log("warmup raised to 3")
        args.warmup = 3
    rank, world, local_rank = dist_env()
    multi = args.workload in MULTI
    if args.workload == "serving":
        if args.impl == "reference":
            run_reference_serving(args, rank, world)
        else:
            run_serving(args, rank, world, local_rank)
        return
    if args.impl == "reference":
        (run_reference_multi if multi else run_reference)(args, rank, world)
    else:
        (run_gb300_multi if multi else run_gb300)(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
