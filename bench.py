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
# pitch 2-4 um, gap 1-3 um) at -m5e-4 -d2 (link tolerance 1e-3): 13,056 to
# 165,888 panels each, 2,193,543 panels, 428 conductors and 318.8M links in
# all (within 32-bit link indices, so one problem holds the whole batch).
MULTI = {
    "crossings32": (lambda: __import__("fastercap_gb300.geometry", fromlist=["x"]).crossing_batch(0, 32, 2, 10),
                    5e-4, 2.0, 1e-4),
}


# DRAM bytes per link-product launch (dram__bytes_read.sum +
# dram__bytes_write.sum) from one ncu capture of the same kernel and
# workload, with the summary that records the capture
LINK_TRAFFIC = {
    "sphere_327680": (534.116864e6 + 4.707072e6, "profiles/sphere_327680_kernels_full.md"),  # k_spmv32<1, 16>
    "crossing8x8_slab": (677.425664e6 + 7.629056e6, "profiles/crossing8x8_slab_spmv32_multi.md"),  # k_spmv32_multi<16>
    "serving_request0": (282.506752e6 + 16.958976e6, "profiles/serving_request0_kernels.md"),  # k_spmv32_multi<24>
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
        "vs_baseline": None, "dtype": "f32 links / f32-pair Krylov", "data": "synthetic",
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


# Serving (the metric's configuration): request r is the input file of
# random_crossing(r) (numpy default_rng(r): k in 2..12, bar length 10-60 um,
# pitch 2-4 um, gap 1-3 um, vacuum); arrivals are Poisson at rate lam with
# inter-arrival times from default_rng(10000 + lam). A request is a whole
# extraction as FasterCap runs one: the server's slot builds the refined mesh
# and the links on the GPU at -m2.5e-4 -d4 (mesh tolerance 2.5e-4, link
# tolerance 1e-3: up to about 400k panels for the largest crossings), fills
# the coefficients and solves every conductor at GMRES tolerance 1e-4 with
# the Jacobi preconditioner. Mixed: FP32 links, all conductors in one batched
# solve; FP64: the plain FP64 path, one right-hand side at a time.
SERVING = {"mesh_eps": 4e-4, "eps_ratio": 2.5, "tol": 1e-4, "kmin": 2, "kmax": 12}
SERVE_ARMS = (("mixed", 1, 0), ("fp64_single_rhs", 0, 1))  # (name, precision, rhs_width)


def serving_config(args):
    """The workload description both arms print (identical dicts)."""
    return {"workload": "serving", "requests": args.requests,
            "rates_req_s": [float(x) for x in args.rates.split(",")],
            "request": "input file of random_crossing(seed = request id): k x k crossing, k in 2..12, length 10-60 um, "
                       "pitch 2-4 um, gap 1-3 um, vacuum; built, filled and solved per request",
            "switches": "-m%g -d%g -t%g -pj" % (SERVING["mesh_eps"], SERVING["eps_ratio"], SERVING["tol"]),
            "link_eps": SERVING["mesh_eps"] * SERVING["eps_ratio"], "gmres_tol": SERVING["tol"], "precond": "jacobi"}


def write_requests(ids, directory):
    from fastercap_gb300 import geometry as geo
    paths = []
    for r in ids:
        path = os.path.join(directory, "req%d.txt" % r)
        geo.random_crossing(int(r), SERVING["kmin"], SERVING["kmax"]).write(path)
        paths.append(path)
    return paths


def arrivals(n_total, lam):
    return np.cumsum(np.random.default_rng(10000 + int(lam)).exponential(1.0 / lam, n_total))


def serve_pass(srv, paths, ids, n_total, precision, rhs_width, lam, world=1):
    """Submit every request of this GPU's shard at its arrival time (one
    Poisson schedule over all n_total requests); per request (latency ms,
    completion s, C, iterations, info)."""
    arr = arrivals(n_total, lam)
    from fastercap_gb300 import replicas
    replicas.barrier(world)
    t0 = time.perf_counter()
    sub = []
    for r, path in zip(ids, paths):
        dt = t0 + arr[r] - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        ts = time.perf_counter()
        sub.append((ts, srv.submit_file(path, precision, tol=SERVING["tol"], mesh_eps=SERVING["mesh_eps"],
                                        eps_ratio=SERVING["eps_ratio"], rhs_width=rhs_width)))
    out = []
    for ts, j in sub:
        cap, it = j.result()
        lat = j.info["queue_ms"] + j.info["run_ms"]
        out.append((lat, ts - t0 + lat / 1000.0, cap, it, j.info))
    return out


def summarize(out, parts, n):
    lat = np.array([x for p_ in parts for x in p_[0]])
    span = max(p_[1] for p_ in parts)
    infos = [o[4] for o in out]
    return {"requests": int(len(lat)), "solves_s": len(lat) / span, "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)),
            "span_s": span, "mean_queue_ms": float(np.mean([i["queue_ms"] for i in infos])),
            "mean_build_ms": float(np.mean([i["build_ms"] for i in infos])),
            "mean_fill_ms": float(np.mean([i["fill_ms"] for i in infos])),
            "mean_solve_ms": float(np.mean([i["solve_ms"] for i in infos]))}


def serving_roofline(ctx, path):
    """Link-product roofline of one request solved resident (mixed, all
    conductors batched): CUDA events around every link-product launch."""
    import fastercap_gb300 as fc
    m = fc.Model.build(path, mesh_eps=SERVING["mesh_eps"], eps_ratio=SERVING["eps_ratio"], ctx=ctx)
    p = ctx.problem(m, fc.PREC_MIXED)
    p.fill()
    p.solve(tol=SERVING["tol"])
    p.reset_stats()
    p.set_profiling(True)
    p.fill()
    p.solve(tol=SERVING["tol"])
    st = p.stats()
    p.close()
    peak, peak_kind = peaks()
    ms = st["link_ms"] / max(1, st["link_launches"])
    b = st["link_bytes"] / max(1, st["link_launches"])
    ach = b / (ms / 1000.0) / 1e9 if ms > 0 else None
    return {"kernel": "k_spmv32_multi (link product)", "bound": "hbm",
            "timing": "CUDA events around every link-product launch of one resident solve of the request",
            "request_panels": m.n_panels, "request_links": m.n_links, "rhs": len(m.conductor_names),
            "achieved": ach, "peak": peak, "unit": "GB/s", "frac": (ach / peak) if ach else None, "peak_source": peak_kind,
            "traffic": LINK_TRAFFIC["serving_request0"][0], "traffic_source": LINK_TRAFFIC["serving_request0"][1],
            "launches": int(st["link_launches"]), "bytes_per_launch": b, "avg_launch_ms": ms,
            "gather_path": "bound by the L1 gather path, not HBM: L1 LSU wavefronts 63.5 pct of peak, issue 60 pct, "
                           "DRAM 12 pct (ncu, " + LINK_TRAFFIC["serving_request0"][1] + ")",
            "krylov": "k_dots and k_update (about 27 pct of the request's device time) run FP32-pair arithmetic "
                      "on a basis stored as FP32 pairs and are bound by HBM: at Arnoldi step 40 they move 1.20 and "
                      "1.22 GB in 210 and 204 us, 0.84 and 0.89 of the measured copy bandwidth (ncu, "
                      + LINK_TRAFFIC["serving_request0"][1] + ")"}


def converged_accuracy(ctx, paths, tol=1e-8):
    """Mixed against FP64 with both solves converged far below the serving
    tolerance: the difference that precision alone makes (at the serving
    tolerance both share the same GMRES truncation error, which dominates
    the small couplings). Per request the largest per-entry difference."""
    import fastercap_gb300 as fc
    errs = []
    for path in paths:
        m = fc.Model.build(path, mesh_eps=SERVING["mesh_eps"], eps_ratio=SERVING["eps_ratio"], ctx=ctx)
        caps = []
        for prec in (fc.PREC_MIXED, fc.PREC_FP64):
            p = ctx.problem(m, prec)
            p.fill()
            caps.append(p.solve(tol=tol)[0])
            p.close()
        errs.append(float(np.max(np.abs(caps[0] - caps[1]) / np.abs(caps[1]))))
    return {"gmres_tol": tol, "requests": len(paths), "max_rel_c_err": max(errs),
            "per_request": [round(e, 9) for e in errs]}


def krylov_accuracy(ctx, paths):
    """The mixed path's Krylov basis in FP32 pairs (the default) against the
    same solve with an FP64 basis (fcg_solve_options.krylov), and both
    against the FP64 solver, at the serving tolerance on the same requests;
    launch-shape measurement off, so every solve is deterministic. Per
    request the largest per-entry difference over the FP64 solver's entry."""
    import fastercap_gb300 as fc
    d_ab, e_pair, e_f64k, it_diff, n_solves = [], [], [], 0, 0
    for path in paths:
        m = fc.Model.build(path, mesh_eps=SERVING["mesh_eps"], eps_ratio=SERVING["eps_ratio"], ctx=ctx)
        res = {}
        for name, prec, kry in (("pair", fc.PREC_MIXED, fc.KRYLOV_PAIR), ("fp64_basis", fc.PREC_MIXED, fc.KRYLOV_FP64),
                                ("fp64", fc.PREC_FP64, fc.KRYLOV_FP64)):
            p = ctx.problem(m, prec)
            p.set_tuning(False)
            p.fill()
            res[name] = p.solve(tol=SERVING["tol"], krylov=kry)
            p.close()
        ref = np.abs(res["fp64"][0])
        d_ab.append(float(np.max(np.abs(res["pair"][0] - res["fp64_basis"][0]) / ref)))
        e_pair.append(float(np.max(np.abs(res["pair"][0] - res["fp64"][0]) / ref)))
        e_f64k.append(float(np.max(np.abs(res["fp64_basis"][0] - res["fp64"][0]) / ref)))
        it_diff += int(np.sum(res["pair"][1] != res["fp64_basis"][1]))
        n_solves += len(res["pair"][1])

    def dist(e):
        return {"median": float(np.median(e)), "p90": float(np.percentile(e, 90)), "max": float(np.max(e))}
    return {"requests": len(paths), "gmres_tol": SERVING["tol"], "pair_vs_fp64_basis": dist(d_ab),
            "vs_fp64_solver": {"pair_basis": dist(e_pair), "fp64_basis": dist(e_f64k)},
            "iteration_counts_differing": it_diff, "solves": n_solves}


def cpu_serving_sample(paths, budget_s, cores, build_in_subprocess=False):
    """The CPU path on a fixed, ordered sample of the requests: per request
    the model build (the host restatement of the reference's parse, mesh
    refinement and link construction; one thread, the same model bit for
    bit), the FP64 fill and the first conductor's GMRES solve, extrapolated
    to the whole request (the reference solves conductors one after another:
    build + fill + n_cond x the first solve); stops after budget_s. Returns
    (solves/s, number of requests, per-request seconds)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from pyoracle import Oracle
    est, t_start = [], time.perf_counter()
    for path in paths:
        arrays, n_cond, build_s = load_request_arrays(path, build_in_subprocess)
        o = Oracle(arrays, threads=cores)
        t0 = time.perf_counter()
        o.fill()
        t1 = time.perf_counter()
        o.solve_rows(0, 1, SERVING["tol"], 1)
        t2 = time.perf_counter()
        est.append(build_s + (t1 - t0) + n_cond * (t2 - t1))
        if time.perf_counter() - t_start > budget_s:
            break
    return len(est) / sum(est), len(est), est


def cpu_sample_subprocess(budget_s):
    """cpu_serving_sample in a fresh process (no CUDA context, no torch and
    its OpenMP runtime next to the oracle's): its cpu_baseline object, or
    the failure."""
    cores = os.cpu_count() or 1
    r = subprocess.run([sys.executable, "-X", "faulthandler", os.path.abspath(__file__), "--cpu-sample", str(budget_s)],
                       stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
    if r.returncode != 0 or not lines:
        log(r.stderr[-2000:])
        return {"value": None, "unit": "solves/s", "cores": cores, "kind": "port",
                "sample": "failed: exit code %d" % r.returncode}
    return json.loads(lines[-1])


def run_cpu_sample(budget_s):
    """--cpu-sample: the serving requests in order through the CPU path for
    about budget_s seconds; prints the cpu_baseline object."""
    from fastercap_gb300 import build as fbuild
    fbuild.build(reference=False)
    tmp = tempfile.mkdtemp()
    cores = os.cpu_count() or 1
    est, n, t_start = [], 0, time.perf_counter()
    while time.perf_counter() - t_start <= budget_s:
        path = write_requests([n], tmp)[0]
        v, _, e = cpu_serving_sample([path], float("inf"), cores)
        est += e
        os.unlink(path)
        n += 1
    import shutil
    shutil.rmtree(tmp, ignore_errors=True)
    print(json.dumps({"value": len(est) / sum(est), "unit": "solves/s", "cores": cores, "kind": "port",
                      "sample": "requests 0..%d in order: host model build + FP64 fill + the first conductor's "
                                "GMRES, extrapolated to every conductor (%.1f s of CPU work)" % (n - 1, sum(est))}),
          flush=True)


def load_request_arrays(path, build_in_subprocess):
    """(model arrays, conductors, host build seconds) of a request file. In a
    subprocess, the CPU arm builds the model there (it writes an .npz with
    the build time), so the arm's own process never loads the GPU library."""
    if not build_in_subprocess:
        import fastercap_gb300 as fc
        t0 = time.perf_counter()
        m = fc.Model.build(path, mesh_eps=SERVING["mesh_eps"], eps_ratio=SERVING["eps_ratio"])
        dt = time.perf_counter() - t0
        # the model's arrays are views of its native storage, freed with it: copy
        arrays = {k: np.array(v, copy=True) for k, v in m.arrays.items()}
        return arrays, int(np.sum(arrays["cond_is_diel"] == 0)), dt
    out = path + ".npz"
    code = ("import sys, time, numpy as np; sys.path.insert(0, %r); import fastercap_gb300 as fc; "
            "t0 = time.perf_counter(); m = fc.Model.build(%r, mesh_eps=%r, eps_ratio=%r); "
            "dt = time.perf_counter() - t0; np.savez(%r, _build_s=np.array(dt), **m.arrays)"
            % (ROOT, path, SERVING["mesh_eps"], SERVING["eps_ratio"], out))
    subprocess.run([sys.executable, "-c", code], check=True)
    d = np.load(out)
    arrays = {k: d[k] for k in d.files if k != "_build_s"}
    build_s = float(d["_build_s"])
    os.unlink(out)
    return arrays, int(np.sum(arrays["cond_is_diel"] == 0)), build_s


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
    tmp = tempfile.mkdtemp()
    ids = replicas.shard(args.requests, rank, world)  # request r is served by GPU r mod world
    paths = write_requests(ids, tmp)
    warm = write_requests(range(10 ** 6, 10 ** 6 + 2 * args.slots), tmp)
    ctx = fc.Context(local_rank)
    res, caps, its = {}, {}, {}
    launches, clk_summary, sizes = 0, None, None
    with ctx.server(slots=args.slots) as srv:
        # warm the pools, the kernels and the tuned launch shapes
        for name, prec, width in SERVE_ARMS:
            for j in [srv.submit_file(p, prec, tol=SERVING["tol"], mesh_eps=SERVING["mesh_eps"],
                                      eps_ratio=SERVING["eps_ratio"], rhs_width=width) for p in warm]:
                j.result()
        for name, prec, width in SERVE_ARMS:
            res[name] = {}
            # the FP64 arm serves the first --fp64-requests of the same arrival
            # schedule (both arms run saturated at the top rate, so their
            # solves/s are the GPU's service rates)
            n_arm = len(ids) if name == "mixed" else sum(1 for r in ids if r < min(args.requests, args.fp64_requests))
            if n_arm == 0:
                continue
            for lam in rates:
                headline = name == "mixed" and lam == rates[-1]
                if headline:
                    with ClockSampler(local_rank) as clk:
                        out = serve_pass(srv, paths[:n_arm], ids[:n_arm], args.requests, prec, width, lam, world)
                    clk_summary = clk.summary()
                else:
                    out = serve_pass(srv, paths[:n_arm], ids[:n_arm], args.requests, prec, width, lam, world)
                # latencies of every GPU's shard; the job ends with the slowest GPU
                parts = replicas.gather_to_all(([o[0] for o in out], max(o[1] for o in out)), world)
                res[name][str(int(lam))] = summarize(out, parts, args.requests)
                caps[(name, lam)] = [o[2] for o in out]
                its[(name, lam)] = [o[3] for o in out]
                if headline:
                    launches = int(sum(o[4]["kernel_launches"] for o in out))
                    sizes = [(o[4]["n_panels"], o[4]["n_links"]) for o in out]
                log("serving %s at %g req/s: %.1f solves/s, p50 %.0f ms, p99 %.0f ms" % (
                    name, lam, res[name][str(int(lam))]["solves_s"], res[name][str(int(lam))]["p50_ms"],
                    res[name][str(int(lam))]["p99_ms"]))
        # latency below saturation: a shorter stream at lower rates (the
        # plain FP64 arm at the lowest one, under its service rate)
        lat_rates = [float(x) for x in args.latency_rates.split(",")] if args.latency_rates else []
        latency = {}
        for name, prec, width in SERVE_ARMS:
            for lam in lat_rates if name == "mixed" else lat_rates[:1]:
                n_arm = sum(1 for r in ids if r < min(args.requests, args.latency_requests))
                if n_arm == 0:
                    continue
                out = serve_pass(srv, paths[:n_arm], ids[:n_arm], args.latency_requests, prec, width, lam, world)
                parts = replicas.gather_to_all(([o[0] for o in out], max(o[1] for o in out)), world)
                latency.setdefault(name, {})[str(int(lam))] = summarize(out, parts, args.latency_requests)
                log("latency %s at %g req/s: %.1f solves/s, p50 %.0f ms, p99 %.0f ms" % (
                    name, lam, latency[name][str(int(lam))]["solves_s"], latency[name][str(int(lam))]["p50_ms"],
                    latency[name][str(int(lam))]["p99_ms"]))
        st = srv.stats()
    top = str(int(rates[-1]))
    # per request: the largest per-entry difference of the mixed matrix from
    # the plain FP64 one, and that entry's size relative to its diagonal
    errs, ent = [], []
    for a, b in zip(caps[("mixed", rates[-1])], caps.get(("fp64_single_rhs", rates[-1]), [])):
        e = np.abs(a - b) / np.abs(b)
        i = np.unravel_index(int(np.argmax(e)), e.shape)
        errs.append(float(e[i]))
        ent.append(float(abs(b[i]) / abs(b[i[0], i[0]])))
    # the same request gives the same matrix at every rate (alone or in any mix)
    same = all(np.array_equal(a, b) for lam in rates for a, b in zip(caps[("mixed", lam)], caps[("mixed", rates[0])]))
    panels = np.array([x[0] for x in sizes])
    links = np.array([x[1] for x in sizes])
    mixed_top = res["mixed"][top]
    lat_top = latency.get("mixed", {}).get(str(int(lat_rates[-1]))) if lat_rates else None
    log("link-product roofline of request 0")
    roof = serving_roofline(ctx, paths[0]) if rank == 0 else None
    log("converged accuracy sample")
    conv = converged_accuracy(ctx, paths[:args.accuracy_sample]) if rank == 0 and args.accuracy_sample > 0 else None
    log("Krylov basis arithmetic sample")
    kry = krylov_accuracy(ctx, paths[:args.krylov_sample]) if rank == 0 and args.krylov_sample > 0 else None
    result = {
        "metric": METRIC, "value": mixed_top["solves_s"], "unit": "solves/s", "n_gpus": world, "steps": args.requests,
        "warmup": 2 * args.slots, "ms_per_step": 1000.0 / mixed_top["solves_s"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 links / f32-pair Krylov", "data": "synthetic",
        # latency under load below the service rate (the highest latency
        # pass); at the top rate every request waits in the queue
        "p50_ms": lat_top["p50_ms"] if lat_top else mixed_top["p50_ms"],
        "p99_ms": lat_top["p99_ms"] if lat_top else mixed_top["p99_ms"],
        "latency_at_req_s": float(lat_rates[-1]) if lat_top else float(rates[-1]),
        "config": serving_config(args),
        "run": {"slots": args.slots, "parallelism": "request r on GPU r mod N" if world > 1 else "single GPU",
                "step": "one request: GPU model build + coefficient fill + GMRES over every conductor + C read back; "
                        "value = mixed solves/s at the highest rate",
                "l2": "no flush: every request builds and uploads its own model (tens to hundreds of MB)",
                "panels_min_max_mean": [int(panels.min()), int(panels.max()), int(panels.mean())],
                "links_min_max_mean": [int(links.min()), int(links.max()), int(links.mean())]},
        "serving": res,
        "latency_below_saturation": latency,
        "mixed_vs_fp64": {"speedup_at_top_rate": mixed_top["solves_s"] / res["fp64_single_rhs"][top]["solves_s"],
                          "max_rel_c_err": max(errs), "requests_compared": len(errs),
                          "requests_above_1e-3": int(sum(e > 1e-3 for e in errs)),
                          "p99_rel_c_err": float(np.percentile(errs, 99)),
                          "worst_entry_over_its_diagonal": ent[int(np.argmax(errs))]} if errs else None,
        "mixed_vs_fp64_converged": conv,
        "mixed_krylov_pair_vs_fp64_basis": kry,
        "same_result_every_rate": bool(same),
        "server": {"max_running": st["max_running"], "peak_in_use_bytes": st["peak_in_use"], "budget_bytes": st["budget"]},
        "e2e": {"value": mixed_top["solves_s"], "unit": "solves/s",
                "h2d_bytes_per_step": int(np.mean([os.path.getsize(p) for p in paths])) + int(
                    np.mean(panels) * 2 * 101 + np.mean(links) * 4),
                "d2h_bytes_per_step": int(np.mean([c.nbytes for c in caps[("mixed", rates[-1])]])),
                "note": "requests arrive as input files on the host; a request's time includes its model build, "
                        "upload and the matrix read back (H2D counts the model arrays problem creation uploads)"},
        "gpu_launches": launches,
        "roofline": roof,
        "clocks": clk_summary,
    }
    if not args.no_cpu_baseline and rank == 0 and world == 1:
        log("CPU sample")
        result["cpu_baseline"] = cpu_sample_subprocess(20.0)
    if args.sphere and rank == 0:
        result["sphere_327680"] = run_gb300(argparse.Namespace(**{**vars(args), "workload": "sphere_327680"}), rank,
                                            world, local_rank, ctx=ctx, emit=False)
    if rank == 0:
        print(json.dumps(result), flush=True)
    ctx.close()
    import shutil
    shutil.rmtree(tmp, ignore_errors=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_request(args):
    """--workload request: one serving request (--request-id) as a server slot
    runs it, for profiling: the input file built on the GPU, then --steps
    resident fills and solves (mixed, all conductors batched, no launch-shape
    measurement), each timed with CUDA events on the problem's stream. Prints
    one JSON line of its own (not the benchmark line)."""
    import fastercap_gb300 as fc
    from fastercap_gb300 import build as fbuild
    fbuild.build(reference=False)
    tmp = tempfile.mkdtemp()
    path = write_requests([args.request_id], tmp)[0]
    ctx = fc.Context(0)
    t0 = time.perf_counter()
    m = fc.Model.build(path, mesh_eps=SERVING["mesh_eps"], eps_ratio=SERVING["eps_ratio"], ctx=ctx)
    build_s = time.perf_counter() - t0
    p = ctx.problem(m, fc.PREC_MIXED)
    p.set_tuning(False)
    times, it, st = [], None, None
    for _ in range(args.steps):
        p.reset_stats()
        t0 = time.perf_counter()
        p.fill()
        cap, it = p.solve(tol=SERVING["tol"])
        times.append(1000.0 * (time.perf_counter() - t0))
        st = p.stats()
    print(json.dumps({"workload": "request", "request_id": args.request_id, "panels": m.n_panels, "links": m.n_links,
                      "conductors": len(m.conductor_names), "gpu_build_s": build_s, "step_ms": times,
                      "fill_ms": st["fill_ms"], "solve_ms": st["solve_ms"], "iterations": [int(x) for x in it],
                      "rhs_width": int(st["rhs_width"]), "kernel_launches": int(st["kernel_launches"])}), flush=True)
    p.close()
    ctx.close()
    import shutil
    shutil.rmtree(tmp, ignore_errors=True)


def run_reference_serving(args, rank, world):
    """CPU arm for serving: the oracle port on every host core, on the
    requests in order (warmup ones first); per step one request's host model
    build, FP64 fill and first conductor's GMRES, extrapolated to all its
    conductors. Models are built in a subprocess (timed there), so this
    process never loads the GPU library."""
    if rank != 0:
        return
    from fastercap_gb300 import build as fbuild
    fbuild.build(reference=False)
    tmp = tempfile.mkdtemp()
    paths = write_requests(range(args.warmup + args.steps), tmp)
    cores = os.cpu_count() or 1
    _, _, est = cpu_serving_sample(paths, float("inf"), cores, build_in_subprocess=True)
    times = est[args.warmup:]
    total = sum(times)
    value = len(times) / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "p50_ms": 1000 * float(np.percentile(times, 50)), "p99_ms": 1000 * float(np.percentile(times, 99)),
        "config": serving_config(args),
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port",
                         "sample": "requests %d..%d in order, one per step: host model build + FP64 fill + the first "
                                   "conductor's GMRES solve, extrapolated to every conductor"
                                   % (args.warmup, args.warmup + args.steps - 1)},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    import shutil
    shutil.rmtree(tmp, ignore_errors=True)
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


def run_gb300(args, rank, world, local_rank, ctx=None, emit=True):
    """One resident workload; prints its line (emit) or returns it (inside
    another workload's run, on that run's context)."""
    import torch
    import fastercap_gb300 as fc
    from fastercap_gb300 import build as fbuild
    own = ctx is None
    if own:
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
        "vs_baseline": None, "dtype": "f32 links / f32-pair Krylov", "data": "synthetic",
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
                     "traffic": LINK_TRAFFIC.get(args.workload, (None, None))[0],
                     "traffic_source": LINK_TRAFFIC.get(args.workload, (None, None))[1], "launches": int(st["link_launches"]),
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
    prob.close()
    if not own:
        return result
    if rank == 0:
        print(json.dumps(result), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="serving", choices=sorted(WORKLOADS) + sorted(MULTI) + ["serving", "request"])
    ap.add_argument("--request-id", type=int, default=0, help="request: which serving request to build and solve")
    ap.add_argument("--requests", type=int, default=2000, help="serving: number of requests")
    ap.add_argument("--rates", default="500", help="serving: arrival rates (req/s), comma separated")
    ap.add_argument("--slots", type=int, default=8, help="serving: concurrent jobs")
    ap.add_argument("--latency-rates", default="5,20",
                    help="serving: arrival rates (req/s) of the shorter latency passes (FP64 arm: the first only)")
    ap.add_argument("--latency-requests", type=int, default=60, help="serving: requests per latency pass")
    ap.add_argument("--fp64-requests", type=int, default=400,
                    help="serving: requests the plain FP64 arm serves (the first ones of the same schedule)")
    ap.add_argument("--accuracy-sample", type=int, default=8,
                    help="serving: requests re-solved at GMRES tolerance 1e-8 in both precisions")
    ap.add_argument("--krylov-sample", type=int, default=40,
                    help="serving: requests solved mixed with the FP32-pair and the FP64 Krylov basis and in FP64")
    ap.add_argument("--no-sphere", dest="sphere", action="store_false",
                    help="serving: skip the resident 327,680-triangle sphere measured after the requests")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-sample", type=float, default=None, help=argparse.SUPPRESS)
    args = ap.parse_args()
    if args.cpu_sample is not None:
        run_cpu_sample(args.cpu_sample)
        return
    if args.warmup < 3:
        log("warmup raised to 3")
        args.warmup = 3
    rank, world, local_rank = dist_env()
    multi = args.workload in MULTI
    if args.workload == "request":
        run_request(args)
        return
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
