"""Edge cases of the solve path: the smallest models (one panel: no links at
all; two panels: one link each way), ragged conductors (one panel next to
hundreds), malformed arrays rejected before any device work, and the
console's handling of the two-level switch.

CPU tests check the model validation that runs before the GPU is touched
(`fcg_model_arrays_check`, the checks `fcg_problem_create` makes first) and
the console's option parsing; GPU tests compare against the oracle."""

import numpy as np
import pytest

import fastercap_gb300 as fc
from conftest import load_golden, model_arrays
from pyoracle import Oracle

ONE_TRIANGLE = """0 one triangle
T c1 0 0 0  1 0 0  0 1 0
"""

TWO_TRIANGLES = """0 two conductors, one triangle each
T a 0 0 0  1 0 0  0 1 0
T b 0 0 2  1 0 2  0 1 2
"""


def write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def one_leaf_model():
    """A model of one leaf panel and no links (the builder always bisects a
    lone panel once, as the reference does, so this one is made by hand)."""
    v = np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float32)
    a = {
        "node_type": np.array([1], np.uint8), "node_left": np.array([-1], np.int32),
        "node_right": np.array([-1], np.int32), "node_leaf_first": np.array([0], np.int64),
        "node_leaf_count": np.array([1], np.int64), "node_vertices": v,
        "node_centroid": v.reshape(1, 3, 3).mean(axis=1).astype(np.float32),
        "node_normal": np.array([[0, 0, 1]], np.float32), "node_area": np.array([0.5]),
        "node_maxside": np.array([np.sqrt(2.0)]), "link_ptr": np.array([0, 0], np.int64),
        "link_src": np.zeros(0, np.int32), "leaf_diel": np.array([0], np.uint8),
        "cond_is_diel": np.array([0], np.uint8), "cond_leaf_first": np.array([0], np.int64),
        "cond_leaf_count": np.array([1], np.int64), "cond_outperm": np.array([1.0]),
        "cond_inperm": np.array([1.0]), "cond_surf_ptr": np.array([0, 1], np.int32),
        "cond_surf_outperm": np.array([1.0]),
    }
    return fc.Model.from_arrays(a)


def test_lone_panel_is_bisected_like_the_reference(tmp_path):
    m = fc.Model.build(write(tmp_path, "one.txt", ONE_TRIANGLE), mesh_eps=1e30, eps_ratio=1e-30)
    assert (m.n_panels, m.n_nodes, m.n_links) == (2, 3, 2)  # the reference's own counts for this input


def test_one_panel_model_has_no_links():
    m = one_leaf_model()
    assert m.n_panels == 1 and m.n_links == 0
    o = Oracle(m.arrays)
    o.fill()
    cap, it, _, _ = o.solve(1e-6, 1)
    assert cap.shape == (1, 1) and cap[0, 0] > 0


@pytest.mark.gpu
def test_one_panel_solve():
    m = one_leaf_model()
    o = Oracle(m.arrays)
    o.fill()
    ocap, oit, _, _ = o.solve(1e-6, 1)
    with fc.Context(0) as ctx:
        for prec in (fc.PREC_FP64, fc.PREC_MIXED):
            p = ctx.problem(m, prec)
            p.fill()
            cap, it = p.solve(tol=1e-6)
            np.testing.assert_allclose(cap, ocap, rtol=1e-12 if prec == fc.PREC_FP64 else 1e-6)
            np.testing.assert_array_equal(it, oit)
            # the product of a model without links is the self term alone
            # (computed in FP32 on the mixed path)
            q = np.array([2.0])
            np.testing.assert_allclose(p.matvec(q), o.matvec(q), rtol=1e-12 if prec == fc.PREC_FP64 else 1e-6)


@pytest.mark.gpu
def test_two_panels_and_ragged_conductors(tmp_path):
    m = fc.Model.build(write(tmp_path, "two.txt", TWO_TRIANGLES), mesh_eps=1e30, eps_ratio=1e-30)
    assert len(m.conductor_names) == 2
    o = Oracle(m.arrays)
    o.fill()
    ocap, oit, _, _ = o.solve(1e-8, 1)
    # one 1-panel geometry next to a large one in the same batch
    g = load_golden("crossing2x2_m02")
    big = fc.Model.from_arrays(model_arrays(g))
    cat, geom = fc.Model.concat([m, big])
    with fc.Context(0) as ctx:
        p = ctx.problem(m, fc.PREC_FP64)
        p.fill()
        cap, it = p.solve(tol=1e-8)
        np.testing.assert_allclose(cap, ocap, rtol=1e-9)
        np.testing.assert_array_equal(it, oit)
        q = ctx.problem(cat, fc.PREC_FP64)
        q.fill()
        q.set_geometries(geom)
        caps, its = q.solve(tol=1e-8)
        np.testing.assert_allclose(caps[0], ocap, rtol=1e-9)
        ob = Oracle(big.arrays)
        ob.fill()
        bcap, bit, _, _ = ob.solve(1e-8, 1)
        np.testing.assert_allclose(caps[1], bcap, rtol=1e-6)
        np.testing.assert_array_equal(its[1], bit)


def _corrupt(key, fn):
    g = load_golden("crossing2x2_m05")
    a = {k: np.array(v, copy=True) for k, v in model_arrays(g).items()}
    fn(a[key])
    return a


@pytest.mark.parametrize("key,fn,msg", [
    ("link_ptr", lambda x: x.__setitem__(-1, x[-1] + 1), "link_ptr"),
    ("node_left", lambda x: x.__setitem__(len(x) - 1, len(x) - 1), "post-order"),
    ("node_leaf_count", lambda x: x.__setitem__(len(x) - 1, x[-1] + 1), "leaf counts"),
    ("cond_leaf_count", lambda x: x.__setitem__(0, x[0] + 1), "tile"),
])
def test_malformed_arrays_rejected(key, fn, msg):
    """The structural checks that fcg_problem_create runs before any device
    work (fcg_model_arrays_check, no GPU needed)."""
    fc.Model.from_arrays(model_arrays(load_golden("crossing2x2_m05"))).check()
    with pytest.raises(fc.FCError) as e:
        fc.Model.from_arrays(_corrupt(key, fn)).check()
    assert msg in str(e.value)


@pytest.mark.gpu
@pytest.mark.parametrize("key,fn,msg", [
    ("link_ptr", lambda x: x.__setitem__(-1, x[-1] + 1), "link_ptr"),
    ("node_left", lambda x: x.__setitem__(len(x) - 1, len(x) - 1), "post-order"),
    ("node_leaf_count", lambda x: x.__setitem__(len(x) - 1, x[-1] + 1), "leaf counts"),
    ("cond_leaf_count", lambda x: x.__setitem__(0, x[0] + 1), "tile"),
])
def test_malformed_arrays_rejected_on_device_context(key, fn, msg):
    with fc.Context(0) as ctx:
        with pytest.raises(fc.FCError) as e:
            ctx.problem(fc.Model.from_arrays(_corrupt(key, fn)), fc.PREC_FP64)
        assert msg in str(e.value)


def test_cli_two_level_switch_parsed(tmp_path):
    """-ps without a number is a command-line error, as in the reference."""
    inp = write(tmp_path, "one.txt", ONE_TRIANGLE)
    assert fc.run_command_line("fastercap_gb300 %s -ps" % inp) == fc.COMMAND_LINE_ERROR


@pytest.mark.parametrize("switch", ["-oi", "-kc"])
def test_cli_refuses_list_file_outputs(tmp_path, switch, capfd):
    """The input-geometry dump and the kept-charge files are not written by
    this solver: their switches are a command-line error, not silently
    dropped."""
    inp = write(tmp_path, "one.txt", ONE_TRIANGLE)
    assert fc.run_command_line("fastercap_gb300 %s %s" % (inp, switch)) == fc.COMMAND_LINE_ERROR
    assert "not written by the GPU solver" in capfd.readouterr().out


@pytest.mark.gpu
def test_cli_two_level_runs(tmp_path, capfd):
    g = load_golden("crossing2x2_m02_ps64")
    inp = tmp_path / "input.txt"
    inp.write_bytes(bytes(g["input_text"]))
    code = fc.run_command_line("fastercap_gb300 %s -m0.02 -t1e-4 -ps64 -x64" % inp)
    out = capfd.readouterr().out
    assert code == fc.NORMAL_END, out
    assert "Two-levels" in out and "Capacitance matrix is:" in out


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["auto_crossing2x2", "auto_crossing2x2_slab"])
def test_cli_auto_mode_matches_reference(name, tmp_path, capfd):
    """-a<err>: the same refinement sequence (panels and links per iteration,
    bit-exact builder) and final matrix as the reference console's own run."""
    import sys
    import os
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    from make_golden import parse_report
    g = load_golden(name)
    inp = tmp_path / "input.txt"
    inp.write_bytes(bytes(g["input_text"]))
    sw = " ".join(str(x) for x in g["switches"])
    code = fc.run_command_line("fastercap_gb300 %s %s -x64 -e" % (inp, sw))
    out = capfd.readouterr().out
    assert code == fc.NORMAL_END, out
    rep = parse_report(out)
    np.testing.assert_array_equal(rep["ref_auto_panels"], g["ref_auto_panels"])
    np.testing.assert_array_equal(rep["ref_auto_links"], g["ref_auto_links"])
    np.testing.assert_allclose(rep["ref_cap"], g["ref_cap"], rtol=2e-5)
    # -e: the matrix as <input>.csv
    csv = np.loadtxt(tmp_path / "input.csv", delimiter=",")
    np.testing.assert_allclose(csv, rep["ref_cap"], rtol=1e-5)


def _compare_list_file(got: str, ref: str, rtol: float, what: str):
    """Line by line, token by token: names and %g coordinates equal as text,
    the trailing %e charge densities within rtol (plus 1e-6 of the file's
    largest density, for densities that nearly cancel)."""
    gl, rl = got.splitlines(), ref.splitlines()
    assert len(gl) == len(rl), what
    dens = [abs(float(ln.split()[-1])) for ln in rl if ln.startswith("T ") and "e" in ln.split()[-1]]
    atol = 1e-6 * max(dens) if dens else 0.0
    for a, b in zip(gl, rl):
        ta, tb = a.split(), b.split()
        assert len(ta) == len(tb), (what, a, b)
        for x, y in zip(ta, tb):
            if "e-" in y or "e+" in y:
                assert abs(float(x) - float(y)) <= rtol * abs(float(y)) + atol, (what, a, b)
            else:
                assert x == y, (what, a, b)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["out_c22", "out_slab"])
@pytest.mark.parametrize("prec,rtol", [("-x64", 1e-5), ("-xm", 2e-3)])
def test_cli_list_files_match_reference(name, prec, rtol, tmp_path, capfd):
    """-o and -c: the same list and panel files as the reference console's
    (CAutoRefine::OutputFastCapFile): names, panel lines in leaf order,
    surfaces, dielectric lines; charge densities within the precision's
    tolerance (FP64 path 1e-5, mixed 2e-3)."""
    import json
    import os
    g = load_golden(name)
    ref = json.loads(bytes(g["files_json"]).decode())
    inp = tmp_path / (name + ".txt")
    inp.write_bytes(bytes(g["input_text"]))
    sw = " ".join(str(x) for x in g["switches"])
    code = fc.run_command_line("fastercap_gb300 %s %s -o -c %s" % (inp, sw, prec))
    out = capfd.readouterr().out
    assert code == fc.NORMAL_END, out
    got = sorted(f for f in os.listdir(tmp_path) if f != inp.name)
    assert got == sorted(ref), out
    for f in ref:
        _compare_list_file((tmp_path / f).read_text(), ref[f], rtol, f)
