"""Serving (fcg_server_*): continuous admission of extraction jobs on one GPU.

Every job's capacitance matrix is the same alone and in a mix of concurrent
jobs (bit for bit: jobs share no state and every kernel sums in a fixed
order), and within the stated tolerance of the oracle's FP64 result (FP64
path 1e-6, mixed path 1e-3 per entry). Admission respects the memory budget
(a budget below every footprint runs one job at a time), queued jobs can be
cancelled, and a cancelled solve returns FCG_USER_BREAK.
"""

import numpy as np
import pytest

import fastercap_gb300 as fc
from fastercap_gb300 import geometry as geo
from pyoracle import Oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = fc.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def models(tmp_path_factory):
    d = tmp_path_factory.mktemp("srv")
    ms = []
    for r in range(6):
        path = d / ("req%d.txt" % r)
        geo.random_crossing(r, kmin=2, kmax=4).write(str(path))
        ms.append(fc.Model.build(str(path), mesh_eps=0.02))
    return ms


def oracle_cap(m, tol):
    o = Oracle(m.arrays)
    o.fill()
    return o.solve(tol, 1)[0]


@pytest.mark.parametrize("precision", [fc.PREC_FP64, fc.PREC_MIXED])
def test_same_alone_and_in_mix(ctx, models, precision):
    with ctx.server(slots=4) as srv:
        alone = []
        for m in models:
            alone.append(srv.submit(m, precision, tol=1e-4).result())
        jobs = [srv.submit(m, precision, tol=1e-4) for m in models + models]
        mixed = [j.result() for j in jobs]
        st = srv.stats()
    assert st["completed"] == 3 * len(models)
    for i, (cap, it) in enumerate(mixed):
        ca, ia = alone[i % len(models)]
        np.testing.assert_array_equal(cap, ca)
        np.testing.assert_array_equal(it, ia)
    tol = 1e-6 if precision == fc.PREC_FP64 else 1e-3
    for m, (cap, _) in zip(models, alone):
        oc = oracle_cap(m, 1e-4)
        assert np.max(np.abs(cap - oc) / np.abs(oc)) < tol


def test_jobs_overlap_with_room(ctx, models):
    with ctx.server(slots=4) as srv:
        jobs = [srv.submit(m, fc.PREC_MIXED, tol=1e-4) for m in models * 3]
        for j in jobs:
            j.result()
        st = srv.stats()
    assert st["max_running"] >= 2
    assert st["in_use"] == 0 and st["running"] == 0


def test_budget_below_footprint_runs_one_at_a_time(ctx, models):
    with ctx.server(slots=4, memory_budget=1) as srv:
        jobs = [srv.submit(m, fc.PREC_MIXED, tol=1e-4) for m in models]
        infos = []
        for j in jobs:
            j.result()
            infos.append(j.info)
        st = srv.stats()
    assert st["max_running"] == 1
    assert all(i["status"] == fc.NORMAL_END for i in infos)
    # footprints cover what the problems held
    assert all(i["device_bytes"] <= i["footprint_bytes"] for i in infos)


def test_cancel_queued_job(ctx, models):
    with ctx.server(slots=1, memory_budget=1) as srv:
        jobs = [srv.submit(m, fc.PREC_FP64, tol=1e-6) for m in models]
        last = jobs[-1]
        last.cancel()
        for j in jobs[:-1]:
            j.result()
        with pytest.raises(fc.FCError) as e:
            last.result()
        assert e.value.code == fc.USER_BREAK
        assert last.info["state"] == fc.JOB_CANCELLED


def test_problem_cancel(ctx, models):
    p = ctx.problem(models[0], fc.PREC_FP64)
    p.fill()
    p.cancel()
    with pytest.raises(fc.FCError) as e:
        p.solve(tol=1e-6)
    assert e.value.code == fc.USER_BREAK


def test_estimate_covers_solve(ctx, models):
    for m in models[:3]:
        p = ctx.problem(m, fc.PREC_MIXED)
        p.fill()
        _, it = p.solve(tol=1e-4)
        assert p.device_bytes <= fc.estimate_bytes(m, fc.PREC_MIXED, iterations=int(it.max()))


def test_failed_job_does_not_stop_the_server(ctx, models):
    """A job whose model is refused fails alone with its status and message;
    the jobs around it complete."""
    from conftest import load_golden, model_arrays
    bad = {k: np.array(v, copy=True) for k, v in model_arrays(load_golden("crossing2x2_m05")).items()}
    bad["link_src"][3] = len(bad["node_type"]) + 7
    with ctx.server(slots=2) as srv:
        jobs = [srv.submit(models[0], fc.PREC_MIXED, tol=1e-4), srv.submit(fc.Model.from_arrays(bad), fc.PREC_MIXED, tol=1e-4),
                srv.submit(models[1], fc.PREC_MIXED, tol=1e-4)]
        jobs[0].result()
        with pytest.raises(fc.FCError) as e:
            jobs[1].result()
        assert "out of range" in str(e.value)
        assert jobs[1].info["state"] == fc.JOB_DONE and jobs[1].info["status"] == fc.GENERIC_ERROR
        jobs[2].result()
        assert srv.stats()["completed"] == 3


def test_file_jobs_equal_model_jobs(ctx, tmp_path):
    """A request given as an input file (the slot builds its model on the GPU)
    gives the matrix of the same model submitted built, bit for bit, alone
    and in a mix with model jobs; a missing file fails alone with the
    builder's status."""
    paths, built = [], []
    for r in range(4):
        path = tmp_path / ("req%d.txt" % r)
        geo.random_crossing(100 + r, kmin=2, kmax=5).write(str(path))
        paths.append(str(path))
        built.append(fc.Model.build(str(path), mesh_eps=0.02, eps_ratio=2.0))
    with ctx.server(slots=3) as srv:
        ref = [srv.submit(m, fc.PREC_MIXED, tol=1e-4).result() for m in built]
        jobs = []
        for p, m in zip(paths, built):
            jobs.append(srv.submit_file(p, fc.PREC_MIXED, tol=1e-4, mesh_eps=0.02, eps_ratio=2.0))
            jobs.append(srv.submit(m, fc.PREC_MIXED, tol=1e-4))
        missing = srv.submit_file(str(tmp_path / "nope.txt"), fc.PREC_MIXED, tol=1e-4)
        out = [j.result() for j in jobs]
        with pytest.raises(fc.FCError) as e:
            missing.result()
        assert e.value.code == fc.CANNOT_OPEN_FILE
        st = srv.stats()
    assert st["in_use"] == 0 and st["running"] == 0
    for i, (cap, it) in enumerate(out):
        np.testing.assert_array_equal(cap, ref[i // 2][0])
        np.testing.assert_array_equal(it, ref[i // 2][1])
    for i in range(0, len(jobs), 2):
        info = jobs[i].info
        assert info["build_ms"] > 0 and info["n_panels"] == built[i // 2].n_panels
        assert info["n_links"] == built[i // 2].n_links


def test_file_jobs_respect_the_budget(ctx, tmp_path):
    """File jobs build first and then wait for memory: with a budget below
    every footprint only one solve holds memory at a time."""
    paths = []
    for r in range(3):
        path = tmp_path / ("req%d.txt" % r)
        geo.random_crossing(200 + r, kmin=2, kmax=4).write(str(path))
        paths.append(str(path))
    with ctx.server(slots=3, memory_budget=1) as srv:
        jobs = [srv.submit_file(p, fc.PREC_FP64, tol=1e-4, mesh_eps=0.05) for p in paths]
        for j in jobs:
            j.result()
        st = srv.stats()
    assert st["completed"] == 3 and st["in_use"] == 0
    assert st["peak_in_use"] <= max(j.info["footprint_bytes"] for j in jobs)
