"""The CPU oracle pinned against the reference solver's own outputs
(tests/golden, produced by the reference compiled from its sources)."""

import numpy as np

import pytest

from conftest import golden_names, load_golden, model_arrays, solve_params, super_dim
from pyoracle import Oracle


def test_fill_matches_reference(golden):
    name, g = golden
    o = Oracle(model_arrays(g))
    coef, selfc = o.fill()
    # same formulas, same operation order: agreement to the last bits
    np.testing.assert_allclose(coef, g["ref_link_coef"], rtol=1e-13, atol=0)
    np.testing.assert_allclose(selfc, g["ref_self_coef"], rtol=1e-13, atol=0)


def test_matvec_matches_reference(golden):
    name, g = golden
    o = Oracle(model_arrays(g))
    for q, v in zip(g["ref_mv_q"], g["ref_mv_v"]):
        out = o.matvec(q, g["ref_link_coef"], g["ref_self_coef"])
        np.testing.assert_array_equal(out, v)


def test_solve_matches_reference(golden):
    name, g = golden
    o = Oracle(model_arrays(g))
    tol, precond = solve_params(g)
    cap, it, _, capped = o.solve(tol, precond, g["ref_link_coef"], g["ref_self_coef"], super_dim(g))
    assert not capped
    np.testing.assert_array_equal(it, g["ref_iterations"])
    np.testing.assert_allclose(cap, g["ref_cap"], rtol=1e-12, atol=0)


def test_sphere_capacitance_near_analytic():
    from conftest import load_golden
    g = load_golden("sphere_d2")
    four_pi_e0_r = 1.1126500559756e-10
    c = g["ref_cap"][0, 0]
    # 320 flat triangles under-resolve the sphere; the error shrinks with refinement
    assert abs(c - four_pi_e0_r) / four_pi_e0_r < 0.02


@pytest.mark.parametrize("name", [n for n in golden_names() if "_ps" in n])
def test_two_level_preconditioner_matches_reference(name):
    """Super elements, leaf map, leaf areas and the inverse super potential
    matrix equal the reference's (same formulas and operation order)."""
    g = load_golden(name)
    o = Oracle(model_arrays(g))
    nodes, index, area, minv = o.super_build(super_dim(g))
    np.testing.assert_array_equal(nodes, g["ref_sup_nodes"])
    np.testing.assert_array_equal(index, g["ref_sup_index"])
    np.testing.assert_array_equal(area, g["ref_sup_area"])
    np.testing.assert_allclose(minv, g["ref_sup_minv"], rtol=1e-12, atol=1e-12 * np.abs(g["ref_sup_minv"]).max())


def test_two_level_disabled_with_many_conductors(tmp_path):
    """At least as many conductors as the dimension: no two-level
    preconditioner (the reference drops it and runs GMRES unpreconditioned)."""
    import fastercap_gb300 as fc
    from fastercap_gb300 import geometry as geo
    path = tmp_path / "c8.txt"
    geo.Crossing(k=8, length=20.0, pitch=2.0, gap=1.0, name="c8").write(str(path))
    m = fc.Model.build(str(path), mesh_eps=0.5)
    o = Oracle(m.arrays)
    o.fill()
    assert o.super_build(16) is None
    assert o.super_build(64) is not None
    c2, i2, _, _ = o.solve(1e-3, 2, super_dim=16)
    c0, i0, _, _ = o.solve(1e-3, 0)
    np.testing.assert_array_equal(c2, c0)
    np.testing.assert_array_equal(i2, i0)


def test_solve_rows_equal_full_solve():
    """A few rows of the matrix (those conductors' solves alone) equal the
    same rows of the full solve."""
    g = load_golden("random3")
    o = Oracle(model_arrays(g))
    o.fill()
    tol, precond = solve_params(g)
    cap, it, _, _ = o.solve(tol, precond)
    rows, rit = o.solve_rows(1, 2, tol, precond)
    np.testing.assert_array_equal(rows, cap[1:3])
    np.testing.assert_array_equal(rit, it[1:3])
