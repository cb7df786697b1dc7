"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle and
the reference's golden outputs.

Tolerances: FP64 path - coefficients within 1e-10 relative plus 1e-13 of
the largest coefficient of the model (dielectric links near their source are
central differences of the analytic potential, where the device's fused
multiply-adds move the cancellation noise; coplanar dielectric links are zero
up to that noise),
matvec 1e-13 relative norm, capacitance 1e-6 relative per entry with the reference's GMRES
iteration counts; mixed path - coefficients within 1e-5 relative plus 2e-6
of the largest coefficient (FP32 quadrature and point formulas in the far
field, the FP32 analytic potential in the near field and for the self terms;
the near-field dielectric links are central differences, where FP32 noise is
amplified about tenfold), matvec 2e-6 relative norm, every capacitance entry
within 1e-3 (0.1 %) of the reference FP64 result."""

import numpy as np
import pytest

import fastercap_gb300 as fc
from conftest import build_from_golden, load_golden, model_arrays, solve_params, super_dim
from pyoracle import Oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = fc.Context(0)
    yield c
    c.close()


def rel_norm(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def check_coef(actual, g, rtol, norm_tol):
    ref = g["ref_link_coef"]
    bound = rtol * np.abs(ref) + norm_tol * np.abs(ref).max()
    bad = np.abs(actual - ref) > bound
    assert not bad.any(), (np.nonzero(bad)[0][:5], actual[bad][:5], ref[bad][:5])


def test_fill_fp64(ctx, golden):
    name, g = golden
    p = ctx.problem(fc.Model.from_arrays(model_arrays(g)), fc.PREC_FP64)
    p.fill()
    lc, sc = p.coefficients()
    check_coef(lc, g, 1e-10, 1e-13)
    np.testing.assert_allclose(sc, g["ref_self_coef"], rtol=1e-12, atol=0)


def test_fill_mixed(ctx, golden):
    name, g = golden
    p = ctx.problem(fc.Model.from_arrays(model_arrays(g)), fc.PREC_MIXED)
    p.fill()
    lc, sc = p.coefficients()
    check_coef(lc, g, 1e-5, 2e-6)
    np.testing.assert_allclose(sc, g["ref_self_coef"], rtol=1e-6, atol=0)


@pytest.mark.parametrize("precision,tol", [(fc.PREC_FP64, 1e-13), (fc.PREC_MIXED, 2e-6)])
def test_matvec(ctx, golden, precision, tol):
    name, g = golden
    p = ctx.problem(fc.Model.from_arrays(model_arrays(g)), precision)
    p.fill()
    for q, v in zip(g["ref_mv_q"], g["ref_mv_v"]):
        assert rel_norm(p.matvec(q), v) < tol
    # batched right-hand sides give the same columns as single ones
    qs = np.random.default_rng(7).uniform(-1, 1, (5, p.n_panels))
    vb = p.matvec(qs)
    for i in range(5):
        assert rel_norm(vb[i], p.matvec(qs[i])) < (1e-15 if precision == fc.PREC_FP64 else 1e-6)


def test_solve_fp64_matches_reference(ctx, golden):
    name, g = golden
    tol, precond = solve_params(g)
    p = ctx.problem(fc.Model.from_arrays(model_arrays(g)), fc.PREC_FP64)
    p.fill()
    cap, it = p.solve(tol=tol, precond=precond, precond_dim=super_dim(g))
    np.testing.assert_allclose(cap, g["ref_cap"], rtol=1e-6, atol=0)
    np.testing.assert_array_equal(it, g["ref_iterations"])


def test_solve_mixed_within_tenth_percent(ctx, golden):
    name, g = golden
    tol, precond = solve_params(g)
    p = ctx.problem(fc.Model.from_arrays(model_arrays(g)), fc.PREC_MIXED)
    p.fill()
    cap, it = p.solve(tol=tol, precond=precond, precond_dim=super_dim(g))
    err = np.abs(cap - g["ref_cap"]) / np.abs(g["ref_cap"])
    assert err.max() < 1e-3, err.max()


def test_krylov_basis_arithmetic(ctx, golden):
    """Mixed path with either Krylov basis arithmetic, FP32 pairs (the
    default) or FP64: every capacitance entry within 0.1 % of the reference,
    iteration counts within one of each other."""
    name, g = golden
    tol, precond = solve_params(g)
    p = ctx.problem(fc.Model.from_arrays(model_arrays(g)), fc.PREC_MIXED)
    p.fill()
    kw = dict(tol=tol, precond=precond, precond_dim=super_dim(g))
    cp, itp = p.solve(krylov=fc.KRYLOV_PAIR, **kw)
    cf, itf = p.solve(krylov=fc.KRYLOV_FP64, **kw)
    for c in (cp, cf):
        err = np.abs(c - g["ref_cap"]) / np.abs(g["ref_cap"])
        assert err.max() < 1e-3, err.max()
    assert np.abs(itp.astype(int) - itf.astype(int)).max() <= 1, (itp, itf)


def test_krylov_pair_converged(ctx):
    """Solved far below the serving tolerance, the FP32-pair basis gives the
    FP64 basis' matrix to 1e-5 of each row's diagonal (the FP32 link
    coefficients, not the basis, set the mixed path's accuracy); FP64
    problems ignore the option (bit-identical), and an unknown value is an
    error."""
    g = load_golden("random3")
    p = ctx.problem(fc.Model.from_arrays(model_arrays(g)), fc.PREC_MIXED)
    p.fill()
    cp, _ = p.solve(tol=1e-8, krylov=fc.KRYLOV_PAIR)
    cf, _ = p.solve(tol=1e-8, krylov=fc.KRYLOV_FP64)
    d = np.abs(np.diag(cf))[:, None]
    assert (np.abs(cp - cf) / d).max() < 1e-5, (np.abs(cp - cf) / d).max()
    with pytest.raises(fc.FCError):
        p.solve(tol=1e-4, krylov=7)
    p64 = ctx.problem(fc.Model.from_arrays(model_arrays(g)), fc.PREC_FP64)
    p64.fill()
    a, ia = p64.solve(tol=1e-6, krylov=fc.KRYLOV_PAIR)
    b, ib = p64.solve(tol=1e-6, krylov=fc.KRYLOV_FP64)
    assert np.array_equal(a, b) and np.array_equal(ia, ib)


def test_builder_to_gpu_end_to_end(ctx, golden, tmp_path):
    """Input file -> host builder -> GPU fill and solve, against the reference."""
    name, g = golden
    tol, precond = solve_params(g)
    m = build_from_golden(g, tmp_path)
    p = ctx.problem(m, fc.PREC_FP64)
    p.fill()
    cap, it = p.solve(tol=tol, precond=precond, precond_dim=super_dim(g))
    np.testing.assert_allclose(cap, g["ref_cap"], rtol=1e-6, atol=0)


def test_oracle_fill_vs_gpu_larger(ctx, tmp_path):
    """A larger mesh than the fixtures: GPU against the oracle."""
    from fastercap_gb300 import geometry as geo
    path = tmp_path / "c2.txt"
    geo.crossing_2x2().write(str(path))
    m = fc.Model.build(str(path), mesh_eps=0.005)
    o = Oracle(m.arrays)
    oc, osc = o.fill()
    p = ctx.problem(m, fc.PREC_FP64)
    p.fill()
    lc, sc = p.coefficients()
    np.testing.assert_allclose(lc, oc, rtol=1e-10, atol=1e-13 * np.abs(oc).max())
    q = np.random.default_rng(1).uniform(-1, 1, m.n_panels)
    assert rel_norm(p.matvec(q), o.matvec(q)) < 1e-13
    cap, it = p.solve(tol=1e-4)
    ocap, oit, _, _ = o.solve(1e-4, 1)
    np.testing.assert_allclose(cap, ocap, rtol=1e-6)
    np.testing.assert_array_equal(it, oit)
    pm = ctx.problem(m, fc.PREC_MIXED)
    pm.fill()
    lm, _ = pm.coefficients()
    np.testing.assert_allclose(lm, oc, rtol=1e-5, atol=2e-6 * np.abs(oc).max())
    capm, _ = pm.solve(tol=1e-4)
    assert np.max(np.abs(capm - ocap) / np.abs(ocap)) < 1e-3


def test_invalid_link_source_rejected(ctx):
    """Out-of-range link sources are found on the device and refused."""
    g = load_golden("crossing2x2_m02")
    a = model_arrays(g)
    bad = dict(a)
    src = np.array(a["link_src"], copy=True)
    src[len(src) // 2] = len(a["node_type"]) + 5
    src[0] = -3
    bad["link_src"] = src
    with pytest.raises(fc.FCError) as e:
        ctx.problem(fc.Model.from_arrays(bad), fc.PREC_FP64)
    assert "out of range" in str(e.value)
    p = ctx.problem(fc.Model.from_arrays(a), fc.PREC_FP64)  # the context still works
    p.fill()


def test_two_level_disabled_with_many_conductors(ctx, tmp_path):
    """With at least as many conductors as the dimension the two-level
    preconditioner is dropped (no preconditioner), as in the reference."""
    from fastercap_gb300 import geometry as geo
    path = tmp_path / "c8.txt"
    geo.Crossing(k=8, length=20.0, pitch=2.0, gap=1.0, name="c8").write(str(path))
    m = fc.Model.build(str(path), mesh_eps=0.5)
    p = ctx.problem(m, fc.PREC_FP64)
    p.fill()
    c2, i2 = p.solve(tol=1e-3, precond=fc.PRECOND_TWO_LEVEL, precond_dim=16)
    c0, i0 = p.solve(tol=1e-3, precond=fc.PRECOND_NONE)
    np.testing.assert_array_equal(c2, c0)
    np.testing.assert_array_equal(i2, i0)
    o = Oracle(m.arrays)
    o.fill()
    c3, i3, _, _ = o.solve(1e-3, 2, super_dim=64)
    c4, i4 = p.solve(tol=1e-3, precond=fc.PRECOND_TWO_LEVEL, precond_dim=64)
    np.testing.assert_allclose(c4, c3, rtol=1e-6)
    np.testing.assert_array_equal(i4, i3)


def test_true_residual_refinement(ctx):
    """Mixed path: after GMRES the true residual b - A x is checked; a solve
    stopped early (iteration cap) is restarted from its current solution and
    ends closer to the converged matrix than without the restarts."""
    g = load_golden("random3")
    o = Oracle(model_arrays(g))
    o.fill()
    ref, _, _, _ = o.solve(1e-8, 1)
    p = ctx.problem(fc.Model.from_arrays(model_arrays(g)), fc.PREC_MIXED)
    p.fill()
    p.reset_stats()
    c0, it0 = p.solve(tol=1e-8, max_iter=3, refine=-1, allow_not_converged=True)
    assert p.stats()["refine_checks"] == 0
    c3, it3 = p.solve(tol=1e-8, max_iter=3, refine=4, allow_not_converged=True)
    st = p.stats()
    assert st["refine_checks"] >= 1 and st["refine_cycles"] >= 1
    assert (it3 > it0).all()
    e0 = np.linalg.norm(c0 - ref) / np.linalg.norm(ref)
    e3 = np.linalg.norm(c3 - ref) / np.linalg.norm(ref)
    assert e3 < 0.5 * e0, (e0, e3)
    # converged solves: the default check finds nothing to refine
    p.reset_stats()
    c, it = p.solve(tol=1e-6)
    st = p.stats()
    assert st["refine_checks"] >= 1 and st["refine_cycles"] == 0
    assert np.max(np.abs(c - ref) / np.abs(ref)) < 1e-3


def test_pinned_model_arrays_same_result(ctx):
    """Problem creation from arrays in pinned host memory (link sources
    uploaded in chunks, each relabelled as it arrives) gives the same
    capacitance matrix and iteration counts as from ordinary memory (one
    staged upload)."""
    torch = pytest.importorskip("torch")
    g = load_golden("crossing2x2_m05")
    arrays = model_arrays(g)
    pinned, keep = {}, []
    for k, v in arrays.items():
        a = np.ascontiguousarray(v)
        t = torch.empty(max(a.nbytes, 1), dtype=torch.uint8, pin_memory=True)
        view = t.numpy()[:a.nbytes].view(a.dtype).reshape(a.shape)
        view[...] = a
        pinned[k] = view
        keep.append(t)
    for prec in (fc.PREC_MIXED, fc.PREC_FP64):
        p1 = ctx.problem(fc.Model.from_arrays(arrays), prec)
        p1.fill()
        c1, it1 = p1.solve(tol=1e-4)
        p2 = ctx.problem(fc.Model.from_arrays(pinned), prec)
        p2.fill()
        c2, it2 = p2.solve(tol=1e-4)
        np.testing.assert_array_equal(c1, c2)
        np.testing.assert_array_equal(it1, it2)
        np.testing.assert_array_equal(p1.coefficients()[0], p2.coefficients()[0])
