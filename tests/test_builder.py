"""The host model builder against the reference: identical panels, nodes,
links (and their order inside every row) and geometry, bit for bit."""

import numpy as np
import pytest

import fastercap_gb300 as fc
from fastercap_gb300 import geometry as geo
from conftest import MODEL_KEYS, build_from_golden, load_golden


def test_builder_bit_exact(golden, tmp_path):
    name, g = golden
    m = build_from_golden(g, tmp_path)
    assert (m.n_panels, m.n_nodes, m.n_links) == tuple(int(x) for x in g["ref_counts"])
    for k in MODEL_KEYS:
        a, b = m.arrays[k], g[k]
        if k == "cond_surf_outperm":
            a = a[: len(b)]
        np.testing.assert_array_equal(np.asarray(a).reshape(b.shape), b, err_msg=k)
    assert list(m.names) == [str(s) for s in g["cond_names"]]
    assert m.info["max_mesh_eps"] == float(g["ref_max_mesh_eps"])


def test_missing_file_status(tmp_path):
    with pytest.raises(fc.FCError) as e:
        fc.Model.build(str(tmp_path / "nope.txt"))
    assert e.value.code == fc.CANNOT_OPEN_FILE


@pytest.mark.parametrize("title", ["0 2D strip", "0 a 2d cross-section", "2D"])
def test_2d_input_refused(tmp_path, title):
    """The first line decides 2D against 3D, as in the reference's reader:
    a 2D input is refused with FC_FILE_ERROR (no 2D solver here), the same
    panels under a 3D title build."""
    body = "T c 0 0 0 1 0 0 0 1 0\nT c 0 0 1 1 0 1 0 1 1\n"
    path = tmp_path / "in.txt"
    path.write_text(title + "\n" + body)
    with pytest.raises(fc.FCError) as e:
        fc.Model.build(str(path))
    assert e.value.code == fc.FILE_ERROR and "2D" in str(e.value)
    path.write_text("0 two plates\n" + body)
    m = fc.Model.build(str(path))
    assert m.n_panels >= 2


def test_empty_file_status(tmp_path):
    p = tmp_path / "empty.txt"
    p.write_text("* nothing here\n")
    with pytest.raises(fc.FCError) as e:
        fc.Model.build(str(p))
    assert e.value.code == fc.FILE_ERROR


def test_complex_permittivity_rejected(tmp_path):
    p = tmp_path / "cplx.txt"
    p.write_text("* lossy\nC c.txt 3.0-j0.02 0 0 0\nEnd\nFile c.txt\nT a 0 0 0 1 0 0 0 1 0\nEnd\n")
    with pytest.raises(fc.FCError) as e:
        fc.Model.build(str(p))
    assert e.value.code == fc.FILE_ERROR


def test_coincident_panels_rejected(tmp_path):
    p = tmp_path / "dup.txt"
    p.write_text("* duplicate panel\nT a 0 0 0 1 0 0 0 1 0\nT a 0 0 0 1 0 0 0 1 0\nT b 0 0 3 1 0 3 0 1 3\n")
    with pytest.raises(fc.FCError):
        fc.Model.build(str(p))


def test_external_subfile(tmp_path):
    """C statements may name files on disk next to the input."""
    (tmp_path / "sq.txt").write_text("* square\nQ s 0 0 0 1 0 0 1 1 0 0 1 0\n")
    (tmp_path / "main.txt").write_text("* two squares\nC sq.txt 1.0 0 0 0\nC sq.txt 1.0 0 0 1\n")
    m = fc.Model.build(str(tmp_path / "main.txt"), mesh_eps=0.05)
    assert m.names == ["g1_s", "g2_s"]
    assert m.n_panels > 4


def test_parallel_panel_read_matches_sequential(tmp_path, monkeypatch):
    """A file of at least 20,000 lines has its panel lines read on all host
    threads before the parse; the model is the same as with the sequential
    read, array for array."""
    from fastercap_gb300 import geometry as geo
    path = tmp_path / "s5.txt"
    geo.write_sphere(str(path), 5)  # 20,480 'T' lines
    par = fc.Model.build(str(path), mesh_eps=1e30, eps_ratio=1e-33)
    monkeypatch.setenv("FCG_PARSE_THREADS", "1")
    seq = fc.Model.build(str(path), mesh_eps=1e30, eps_ratio=1e-33)
    assert par.n_panels == seq.n_panels == 20480
    for k in par.arrays:
        np.testing.assert_array_equal(np.asarray(par.arrays[k]), np.asarray(seq.arrays[k]), err_msg=k)


def test_array_views_outlive_model(tmp_path):
    """A built model's arrays are views of its native storage; they keep it
    alive after the Model is closed and dropped."""
    import gc

    path = str(tmp_path / "c.txt")
    geo.crossing_2x2().write(path)
    m = fc.Model.build(path, mesh_eps=0.05)
    src, ptr = m.arrays["link_src"], m.arrays["link_ptr"]
    expect = (src.copy(), ptr.copy())
    m.close()
    del m
    gc.collect()
    churn = [bytearray(1 << 20) for _ in range(64)]
    np.testing.assert_array_equal(src, expect[0])
    np.testing.assert_array_equal(ptr, expect[1])
    del churn


def test_parallel_flatten_same_model(tmp_path, monkeypatch):
    """A model large enough for the multi-threaded flatten (70k nodes, 18
    conductors) is the same, array for array, as the single-threaded one."""
    path = str(tmp_path / "r.txt")
    geo.random_crossing(4, 2, 12).write(path)
    monkeypatch.setenv("FCG_HOST_THREADS", "1")
    a = fc.Model.build(path, mesh_eps=1e-3)
    monkeypatch.delenv("FCG_HOST_THREADS")
    b = fc.Model.build(path, mesh_eps=1e-3)
    assert a.n_nodes >= 50000
    for k in MODEL_KEYS:
        np.testing.assert_array_equal(np.asarray(a.arrays[k]), np.asarray(b.arrays[k]), err_msg=k)
    assert list(a.names) == list(b.names)
