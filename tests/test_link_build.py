"""Link construction on the GPU (fcg_model_build_on) against the host model
builder: the same model bit for bit — every node array, the link rows, the
order of the links inside every row — and the same statistics (recursion
level, achieved mesh refinement). The host builder is itself pinned to the
reference's own arrays on the golden inputs, so the golden cases also compare
the device rows with the reference's directly.

Cases: every golden input (conductors, dielectric interfaces, two-level
switches), a random bus crossing, the 8x8 crossing in a dielectric slab
(dielectric criteria, 16 conductors, 81M links) and a refined sphere (one
conductor, 20,480 panels, deep self traversal)."""

import numpy as np
import pytest

import fastercap_gb300 as fc
from fastercap_gb300 import geometry as geo
from conftest import MODEL_KEYS, load_golden, golden_names, switch_value

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = fc.Context(0)
    yield c
    c.close()


def assert_same_model(dev, host):
    assert dev.info == host.info
    assert list(dev.names) == list(host.names)
    for k in MODEL_KEYS:
        np.testing.assert_array_equal(dev.arrays[k], host.arrays[k], err_msg=k)


def build_pair(ctx, path, **kw):
    return fc.Model.build(path, ctx=ctx, **kw), fc.Model.build(path, **kw)


@pytest.mark.parametrize("name", golden_names())
def test_golden_inputs(ctx, name, tmp_path):
    g = load_golden(name)
    inp = tmp_path / "input.txt"
    inp.write_bytes(bytes(g["input_text"]))
    sw = [str(s) for s in g["switches"]]
    kw = dict(mesh_eps=switch_value(sw, "-m", 0.1), eps_ratio=switch_value(sw, "-d", 1.0))
    dev, host = build_pair(ctx, str(inp), **kw)
    assert_same_model(dev, host)
    # the reference's own rows
    np.testing.assert_array_equal(dev.arrays["link_ptr"], g["link_ptr"])
    np.testing.assert_array_equal(dev.arrays["link_src"], g["link_src"])


def test_random_crossing(ctx, tmp_path):
    p = str(tmp_path / "x.txt")
    geo.random_crossing(3, kmin=4, kmax=6).write(p)
    assert_same_model(*build_pair(ctx, p, mesh_eps=0.02))


def test_dielectric_slab_crossing(ctx, tmp_path):
    p = str(tmp_path / "slab.txt")
    geo.crossing_8x8_slab().write(p)
    dev, host = build_pair(ctx, p, mesh_eps=5e-6, eps_ratio=1.0)
    assert dev.n_links > 50_000_000
    assert_same_model(dev, host)


def test_sphere(ctx, tmp_path):
    p = str(tmp_path / "s.txt")
    geo.write_sphere(p, 5)
    dev, host = build_pair(ctx, p, mesh_eps=1e30, eps_ratio=1e-33)
    assert dev.n_panels == 20480
    assert_same_model(dev, host)


def test_lone_panel(ctx, tmp_path):
    """A lone panel is bisected once; its two halves link each other."""
    p = tmp_path / "one.txt"
    p.write_text("0 one triangle\nT c1 0 0 0  1 0 0  0 1 0\n")
    dev, host = build_pair(ctx, str(p), mesh_eps=1e30, eps_ratio=1e-30)
    assert (dev.n_panels, dev.n_nodes, dev.n_links) == (2, 3, 2)
    assert_same_model(dev, host)


def test_solve_on_device_built_model(ctx, tmp_path):
    """The device-built model solves to the host-built model's matrix (the
    same arrays, so the same FP64 result bit for bit)."""
    p = str(tmp_path / "x.txt")
    geo.random_crossing(5, kmin=2, kmax=3).write(p)
    dev, host = build_pair(ctx, p, mesh_eps=0.05)
    caps = []
    for m in (dev, host):
        pr = ctx.problem(m, fc.PREC_FP64)
        pr.fill()
        caps.append(pr.solve(tol=1e-6)[0])
    np.testing.assert_array_equal(caps[0], caps[1])


def test_touching_conductors(ctx, tmp_path):
    """Two conductors sharing an edge: the refinement recurses towards the
    contact; the device closure reaches the host's mesh (or its error)."""
    p = tmp_path / "touch.txt"
    p.write_text("0 touching\nT a 0 0 0  1 0 0  0 1 0\nT b 1 0 0  0 1 0  1 1 0.5\n")
    results = []
    for c in (ctx, None):
        try:
            m = fc.Model.build(str(p), mesh_eps=0.05, ctx=c)
            results.append(("ok", m))
        except fc.FCError as e:
            results.append(("err", e.code))
    assert results[0][0] == results[1][0]
    if results[0][0] == "ok":
        assert_same_model(results[0][1], results[1][1])
    else:
        assert results[0][1] == results[1][1]


@pytest.mark.parametrize("meps", [0.2, 0.05, 0.01])
def test_mesh_refinement_levels(ctx, tmp_path, meps):
    """Refinement from coarse to fine on a crossing: the mesh (panel count,
    node tree, max achieved refinement value) matches at every setting."""
    p = str(tmp_path / "x.txt")
    geo.random_crossing(11, kmin=3, kmax=3).write(p)
    dev, host = build_pair(ctx, p, mesh_eps=meps)
    assert dev.info["max_mesh_eps"] == host.info["max_mesh_eps"]
    assert_same_model(dev, host)


def test_super_hierarchy_sphere_81920(ctx, tmp_path):
    """81,920 input panels: the super hierarchy is built on the device (every
    set of at least 20,000 panels); the same tree and super nodes as the host
    recursion, so the same model bit for bit."""
    p = str(tmp_path / "s6.txt")
    geo.write_sphere(p, 6)
    dev, host = build_pair(ctx, p, mesh_eps=1e30, eps_ratio=1e-33)
    assert dev.n_panels == 81920
    assert_same_model(dev, host)


def test_super_hierarchy_dielectric_shell(ctx, tmp_path):
    """A conductor sphere inside a dielectric shell (40,960 input panels, the
    shell's super nodes dielectric): device and host super hierarchies agree."""
    V1, T1 = geo.icosphere(5, 1.0)
    V2, T2 = geo.icosphere(5, 2.0)
    lines = ["* conductor sphere in a dielectric shell", "C c.txt  3.9  0.0 0.0 0.0",
             "D d.txt  1.0 3.9  0.0 0.0 0.0  0.0 0.0 3.0", "End", "File c.txt"]
    for a, b, c in T1:
        lines.append("T ball  %.9e %.9e %.9e  %.9e %.9e %.9e  %.9e %.9e %.9e" % (*V1[a], *V1[b], *V1[c]))
    lines += ["End", "File d.txt"]
    for a, b, c in T2:
        lines.append("T shell  %.9e %.9e %.9e  %.9e %.9e %.9e  %.9e %.9e %.9e" % (*V2[a], *V2[b], *V2[c]))
    lines.append("End")
    p = tmp_path / "shell.txt"
    p.write_text("\n".join(lines) + "\n")
    dev, host = build_pair(ctx, str(p), mesh_eps=1e30, eps_ratio=1e-33)
    assert dev.n_panels == 40960
    assert_same_model(dev, host)
