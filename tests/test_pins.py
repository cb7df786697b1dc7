"""Parity at the benchmark configurations' own sizes, against the reference.

tests/golden/pin_*.npz come from the reference solver itself (its own
Solver/*.cpp compiled here, driven by oracle/ref_dump.cpp through
tests/golden/make_golden.py) on:

* pin_crossing2x2_5k - the 2x2 bus crossing (1x1x10 um bars, 3 um pitch,
  layers 1 um apart, vacuum) at -m0.0018 -t1e-4 -pj: 5,088 panels, 10,172
  nodes, 1,369,588 links, four conductors;
* pin_sphere_20480 - the R = 1 m sphere, icosahedron subdivided 5 times,
  -m1e30 -d1e-33 -t1e-4 -pj: 20,480 panels, 40,959 nodes, 4,175,890 links.

Each fixture holds the SHA-256 of every model array in the C-ABI layout (so
the model must be identical bit for bit, link order included), the self
coefficients, every 97th link coefficient, one seeded product, the GMRES
iteration counts and the capacitance matrix.

Tolerances as in test_gpu_parity: FP64 coefficients within 1e-10 relative
plus 1e-13 of the largest, self terms 1e-12, product 1e-13 relative norm,
capacitance 1e-6 per entry with the reference's iteration counts; mixed
coefficients within 1e-5 plus 2e-6 of the largest, product 2e-6, every
capacitance entry within 1e-3 (0.1 %). The CPU oracle port is held to the
reference's own bits (coefficients 1e-13, identical product, same
iterations, capacitance 1e-12).
"""

import hashlib
import os

import numpy as np
import pytest

import fastercap_gb300 as fc
from conftest import GOLDEN, MODEL_KEYS
from fastercap_gb300 import geometry as geo

# input generators of the pinned cases (the fixture stores the input's SHA-256)
PIN_INPUTS = {
    "pin_crossing2x2_5k": lambda: geo.crossing_2x2().text(),
    "pin_sphere_20480": lambda: geo.sphere_text(5),
}
PINS = sorted(PIN_INPUTS)


def load_pin(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: d[k] for k in d.files}


def array_sha256(a) -> str:
    """SHA-256 of an array's dtype, shape and little-endian bytes (the
    generator's definition, tests/golden/make_golden.py)."""
    a = np.ascontiguousarray(a)
    h = hashlib.sha256()
    h.update(("%s|%s|" % (a.dtype.newbyteorder("<").str, ",".join(str(x) for x in a.shape))).encode())
    h.update(a.astype(a.dtype.newbyteorder("<"), copy=False).tobytes())
    return h.hexdigest()


def switch(sw, prefix, default):
    for s in sw:
        if s.startswith(prefix) and not (prefix == "-m" and s.startswith("-mc")):
            return float(s[len(prefix):])
    return default


def write_input(name, g, tmp_path):
    text = PIN_INPUTS[name]()
    assert hashlib.sha256(text.encode()).hexdigest() == str(g["input_sha256"]), "input generator changed"
    path = tmp_path / (name + ".txt")
    path.write_text(text)
    return str(path)


def build(name, g, tmp_path, ctx=None):
    sw = [str(s) for s in g["switches"]]
    return fc.Model.build(write_input(name, g, tmp_path), mesh_eps=switch(sw, "-m", 0.1),
                          eps_ratio=switch(sw, "-d", 1.0), ctx=ctx)


def assert_model_identical(m, g):
    assert (m.n_panels, m.n_nodes, m.n_links) == tuple(int(x) for x in g["ref_counts"])
    want = dict(s.split(":", 1) for s in (str(x) for x in g["model_sha256"]))
    assert sorted(want) == sorted(MODEL_KEYS)
    for k in MODEL_KEYS:
        a = np.asarray(m.arrays[k])
        if k == "cond_surf_outperm" and array_sha256(a) != want[k]:
            # the builder may keep spare room at the end of this array
            a = a[: int(np.asarray(m.arrays["cond_surf_ptr"])[-1])] if len(a) else a
        assert array_sha256(a) == want[k], k
    assert list(m.names) == [str(s) for s in g["cond_names"]]
    assert m.info["max_mesh_eps"] == float(g["ref_max_mesh_eps"])


def solve_tol(g):
    return switch([str(s) for s in g["switches"]], "-t", 0.01)


def check_coef_sample(lc, sc, g, rtol, norm_tol, self_rtol):
    ref = g["ref_link_coef_sample"]
    got = lc[g["ref_link_coef_index"]]
    bound = rtol * np.abs(ref) + norm_tol * np.abs(ref).max()
    bad = np.abs(got - ref) > bound
    assert not bad.any(), (np.nonzero(bad)[0][:5], got[bad][:5], ref[bad][:5])
    np.testing.assert_allclose(sc, g["ref_self_coef"], rtol=self_rtol, atol=0)


def rel_norm(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


# ---------------------------------------------------------------- CPU


@pytest.mark.parametrize("name", PINS)
def test_host_builder_matches_reference_at_size(name, tmp_path):
    g = load_pin(name)
    assert_model_identical(build(name, g, tmp_path), g)


@pytest.mark.parametrize("name", PINS)
def test_oracle_matches_reference_at_size(name, tmp_path):
    """The CPU restatement on the reference's own model: same coefficients,
    the same product bit for bit, the same iterations and matrix."""
    from pyoracle import Oracle
    g = load_pin(name)
    m = build(name, g, tmp_path)
    o = Oracle(m.arrays, threads=os.cpu_count() or 1)
    coef, selfc = o.fill()
    np.testing.assert_allclose(coef[g["ref_link_coef_index"]], g["ref_link_coef_sample"], rtol=1e-13, atol=0)
    np.testing.assert_allclose(selfc, g["ref_self_coef"], rtol=1e-13, atol=0)
    for q, v in zip(g["ref_mv_q"], g["ref_mv_v"]):
        np.testing.assert_array_equal(o.matvec(q, coef, selfc), v)
    cap, it, _, _ = o.solve(solve_tol(g), 1, coef, selfc)
    np.testing.assert_array_equal(np.asarray(it), g["ref_iterations"])
    np.testing.assert_allclose(cap, g["ref_cap"], rtol=1e-12, atol=0)


# ---------------------------------------------------------------- GPU


@pytest.fixture(scope="module")
def ctx():
    c = fc.Context(0)
    yield c
    c.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", PINS)
def test_device_builder_matches_reference_at_size(ctx, name, tmp_path):
    g = load_pin(name)
    assert_model_identical(build(name, g, tmp_path, ctx=ctx), g)


@pytest.mark.gpu
@pytest.mark.parametrize("name", PINS)
def test_fp64_path_matches_reference_at_size(ctx, name, tmp_path):
    g = load_pin(name)
    m = build(name, g, tmp_path, ctx=ctx)
    p = ctx.problem(m, fc.PREC_FP64)
    p.fill()
    lc, sc = p.coefficients()
    check_coef_sample(lc, sc, g, 1e-10, 1e-13, 1e-12)
    for q, v in zip(g["ref_mv_q"], g["ref_mv_v"]):
        assert rel_norm(p.matvec(q), v) < 1e-13
    cap, it = p.solve(tol=solve_tol(g))
    np.testing.assert_array_equal(np.asarray(it), g["ref_iterations"])
    np.testing.assert_allclose(cap, g["ref_cap"], rtol=1e-6, atol=0)
    p.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", PINS)
def test_mixed_path_within_tenth_percent_at_size(ctx, name, tmp_path):
    g = load_pin(name)
    m = build(name, g, tmp_path, ctx=ctx)
    p = ctx.problem(m, fc.PREC_MIXED)
    p.fill()
    lc, sc = p.coefficients()
    check_coef_sample(lc, sc, g, 1e-5, 2e-6, 1e-6)
    for q, v in zip(g["ref_mv_q"], g["ref_mv_v"]):
        assert rel_norm(p.matvec(q), v) < 2e-6
    cap, it = p.solve(tol=solve_tol(g))
    err = np.abs(cap - g["ref_cap"]) / np.abs(g["ref_cap"])
    assert err.max() < 1e-3, err.max()
    p.close()
