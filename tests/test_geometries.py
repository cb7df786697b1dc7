"""Many independent geometries in one problem (fcg_model_concat +
fcg_problem_set_geometries): every geometry keeps its own GMRES solves while
each kernel runs once over all of them.

CPU: the native concatenation and the numpy one agree; the oracle's
coefficients on a concatenation are the per-geometry coefficients one after
another (no link crosses a geometry).
GPU: the batched solve of a concatenation gives, geometry by geometry, the
oracle's capacitance matrices (FP64: 1e-6 relative, equal iteration counts;
mixed: 1e-3) and rejects geometry maps that links or tree edges cross.
"""

import numpy as np
import pytest

import fastercap_gb300 as fc
from conftest import load_golden, model_arrays
from pyoracle import Oracle
from fastercap_gb300 import geometry as geo

GOLDEN_MIX = ["crossing2x2_m02", "sphere_d2", "random3", "crossing2x2_slab", "merged_cubes"]


def golden_models():
    return [fc.Model.from_arrays(model_arrays(load_golden(n))) for n in GOLDEN_MIX]


def oracle_solve(m, tol, precond):
    o = Oracle(m.arrays)
    o.fill()
    return o.solve(tol, precond)


def built_models(tmp_path, seeds=(1, 2, 5)):
    ms = []
    for s in seeds:
        path = tmp_path / ("r%d.txt" % s)
        geo.random_crossing(s, kmin=2, kmax=4).write(str(path))
        ms.append(fc.Model.build(str(path), mesh_eps=0.05))
    return ms


def test_concat_native_matches_numpy(tmp_path):
    ms = built_models(tmp_path)
    native, gn = fc.Model.concat(ms)
    ref, gr = fc.Model._concat_arrays(ms)
    np.testing.assert_array_equal(gn, gr)
    for k in model_arrays(ref.arrays):
        np.testing.assert_array_equal(np.asarray(native.arrays[k]), np.asarray(ref.arrays[k]), err_msg=k)
    assert native.names == ref.names


def test_concat_oracle_block_diagonal():
    ms = golden_models()
    cat, geom = fc.Model.concat(ms)
    assert cat.n_panels == sum(m.n_panels for m in ms)
    assert list(np.bincount(geom)) == [len(m.arrays["cond_is_diel"]) for m in ms]
    oc, osc = Oracle(cat.arrays).fill()
    lo = so = 0
    for m in ms:
        c, sc = Oracle(m.arrays).fill()
        np.testing.assert_array_equal(oc[lo:lo + len(c)], c)
        np.testing.assert_array_equal(osc[so:so + len(sc)], sc)
        lo += len(c)
        so += len(sc)


@pytest.fixture(scope="module")
def ctx():
    c = fc.Context(0)
    yield c
    c.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precond", [1, 0])
def test_segmented_solve_fp64_matches_oracle(ctx, precond):
    ms = golden_models()
    cat, geom = fc.Model.concat(ms)
    p = ctx.problem(cat, fc.PREC_FP64)
    p.fill()
    p.set_geometries(geom)
    caps, its = p.solve(tol=1e-4, precond=precond)
    assert len(caps) == len(ms)
    for m, cap, it in zip(ms, caps, its):
        ocap, oit, _, _ = oracle_solve(m, 1e-4, precond)
        np.testing.assert_allclose(cap, ocap, rtol=1e-6, atol=0)
        np.testing.assert_array_equal(it, oit)


@pytest.mark.gpu
def test_segmented_solve_mixed(ctx):
    ms = golden_models()
    cat, geom = fc.Model.concat(ms)
    p = ctx.problem(cat, fc.PREC_MIXED)
    p.fill()
    p.set_geometries(geom)
    caps, _ = p.solve(tol=1e-4)
    for m, cap in zip(ms, caps):
        ocap, _, _, _ = oracle_solve(m, 1e-4, 1)
        assert np.max(np.abs(cap - ocap) / np.abs(ocap)) < 1e-3


@pytest.mark.gpu
def test_segmented_equals_separate_problems(ctx, tmp_path):
    """Same iterations and matrices as one problem per geometry."""
    ms = built_models(tmp_path, seeds=(3, 4, 6, 7))
    cat, geom = fc.Model.concat(ms)
    p = ctx.problem(cat, fc.PREC_FP64)
    p.fill()
    p.set_geometries(geom)
    caps, its = p.solve(tol=1e-5)
    for m, cap, it in zip(ms, caps, its):
        q = ctx.problem(m, fc.PREC_FP64)
        q.fill()
        c1, i1 = q.solve(tol=1e-5)
        np.testing.assert_allclose(cap, c1, rtol=1e-9)
        np.testing.assert_array_equal(it, i1)


@pytest.mark.gpu
def test_many_columns_batches(ctx, tmp_path):
    """A geometry with more than 32 conductors runs in column batches."""
    path = tmp_path / "c18.txt"
    geo.Crossing(k=18, length=40.0, pitch=2.0, gap=1.0, name="c18").write(str(path))
    m = fc.Model.build(str(path), mesh_eps=0.2)
    assert len(m.conductor_names) == 36
    small = ms = built_models(tmp_path, seeds=(1,))
    cat, geom = fc.Model.concat([m] + ms)
    p = ctx.problem(cat, fc.PREC_FP64)
    p.fill()
    p.set_geometries(geom)
    caps, its = p.solve(tol=1e-3)
    for mm, cap, it in zip([m] + small, caps, its):
        ocap, oit, _, _ = oracle_solve(mm, 1e-3, 1)
        np.testing.assert_allclose(cap, ocap, rtol=1e-6)
        np.testing.assert_array_equal(it, oit)


@pytest.mark.gpu
def test_iteration_cap_per_geometry(ctx):
    """A capped solve stops at its own cap and reports NOT_CONVERGED."""
    ms = golden_models()[:2]
    cat, geom = fc.Model.concat(ms)
    p = ctx.problem(cat, fc.PREC_FP64)
    p.fill()
    p.set_geometries(geom)
    caps, its = p.solve(tol=1e-14, max_iter=3, allow_not_converged=True)
    for it in its:
        assert (it <= 3).all()
    with pytest.raises(fc.FCError):
        p.solve(tol=1e-14, max_iter=3)


@pytest.mark.gpu
def test_geometry_map_rejected(ctx):
    g = load_golden("crossing2x2_m02")
    m = fc.Model.from_arrays(model_arrays(g))
    p = ctx.problem(m, fc.PREC_FP64)
    p.fill()
    nc = len(m.arrays["cond_is_diel"])
    # links join the conductors of one geometry: splitting them is refused
    with pytest.raises(fc.FCError):
        p.set_geometries([0] * (nc // 2) + [1] * (nc - nc // 2))
    with pytest.raises(fc.FCError):
        p.set_geometries([1] * nc)
    with pytest.raises(fc.FCError):
        p.set_geometries([0, 2] + [2] * (nc - 2))
    # the problem still solves as one geometry
    p.set_geometries([0] * nc)
    caps, its = p.solve(tol=1e-4)
    assert len(caps) == 1 and caps[0].shape == (nc, nc)


@pytest.mark.gpu
def test_rhs_width_one_matches_batched(ctx):
    g = load_golden("random3")
    m = fc.Model.from_arrays(model_arrays(g))
    p = ctx.problem(m, fc.PREC_FP64)
    p.fill()
    c1, i1 = p.solve(tol=1e-5, rhs_width=1)
    c2, i2 = p.solve(tol=1e-5)
    np.testing.assert_allclose(c1, c2, rtol=1e-10)
    np.testing.assert_array_equal(i1, i2)
    assert p.charges().shape == (len(m.conductor_names), m.n_panels)
