"""Generate the golden fixtures in tests/golden from the reference solver.

Runs where the reference source tree is present: builds oracle/_ref (the
reference's own Solver/*.cpp compiled against oracle/shim, see
oracle/Makefile), writes each input with fastercap_gb300.geometry, runs
oracle/_ref/fcref_dump on it and packs the dump into <case>.npz:

  input_text            the exact input file (bytes)
  switches              the reference command-line switches used
  model arrays          the reference's post-order node array, links and
                        conductor data converted to the C-ABI layout
  ref_link_coef, ref_self_coef   the reference's FP64 coefficients
  ref_mv_q, ref_mv_v    seeded matrix-vector products through the reference
  ref_cap               the reference's capacitance matrix
  ref_iterations        GMRES Arnoldi steps per conductor
  ref_counts            panels, nodes, links; ref_max_mesh_eps

  ref_sup_*             (two-level cases) the reference's super elements,
                        leaf map, leaf areas and inverse super matrix

Cases named pin_* are kept compact (hashes of the model arrays, a sample of
the link coefficients; see PIN_CASES); auto_* cases come from the reference
console's report.

Usage: python tests/golden/make_golden.py [reference dir [case ...]]
  (an empty reference dir "" takes FCG_REFERENCE_DIR or oracle/Makefile's default)
"""

from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from fastercap_gb300 import geometry as geo  # noqa: E402

TWO_CUBES_MERGED = """* two unit cubes short-circuited with '+', then renamed with N
C cube.txt  1.0  0.0 0.0 0.0 +
C cube.txt  1.0  2.5 0.0 0.0
C bar.txt  1.0  0.0 3.0 0.0
End
File cube.txt
* unit cube
%s
End
File bar.txt
* a bar whose panels use two names, merged by N
%s
N barA barB
End
"""


def _cube_text():
    from fastercap_gb300.geometry import box_faces, _q_line
    return "\n".join(_q_line("cube", f) for f in box_faces(0, 0, 0, 1, 1, 1))


def _bar_text():
    from fastercap_gb300.geometry import box_faces, _q_line
    faces = box_faces(0, 0, 0, 4, 1, 1)
    return "\n".join(_q_line("barA" if i < 3 else "barB", f) for i, f in enumerate(faces))


CASES = {
    # name: (input text factory, switches)
    "crossing2x2_m05": (lambda: geo.crossing_2x2().text(), ["-m0.05", "-t1e-4", "-pj", "-f0"]),
    "crossing2x2_m02": (lambda: geo.crossing_2x2().text(), ["-m0.02", "-t1e-4", "-pj", "-f0"]),
    "crossing2x2_m02_nopc": (lambda: geo.crossing_2x2().text(), ["-m0.02", "-t1e-3", "-pn", "-f0"]),
    "sphere_d2": (lambda: geo.sphere_text(2), ["-m1e30", "-d1e-32", "-t1e-4", "-pj", "-f0"]),
    "crossing2x2_slab": (lambda: geo.Crossing(k=2, length=10.0, pitch=3.0, gap=1.0, eps_r=3.9,
                                              slab=(3.5, 1.0, 3.9, 15.0), name="c2slab").text(),
                         ["-m0.02", "-t1e-4", "-pj", "-f0"]),
    "random3": (lambda: geo.random_crossing(3).text(), ["-m0.05", "-t1e-4", "-pj", "-f0"]),
    "merged_cubes": (lambda: TWO_CUBES_MERGED % (_cube_text(), _bar_text()), ["-m0.05", "-t1e-4", "-pj", "-f0"]),
    # two-level preconditioner (-ps<dim>): conductors only, and with a dielectric interface
    "crossing2x2_m02_ps64": (lambda: geo.crossing_2x2().text(), ["-m0.02", "-t1e-4", "-ps64", "-f0"]),
    "crossing2x2_slab_ps32": (lambda: geo.Crossing(k=2, length=10.0, pitch=3.0, gap=1.0, eps_r=3.9,
                                                   slab=(3.5, 1.0, 3.9, 15.0), name="c2slab").text(),
                              ["-m0.02", "-t1e-4", "-ps32", "-f0"]),
    "sphere_d2_ps256": (lambda: geo.sphere_text(2), ["-m1e30", "-d1e-32", "-t1e-4", "-ps256", "-f0"]),
}


def convert(dump: str) -> dict:
    L = lambda n: np.load(os.path.join(dump, n + ".npy"))
    meta = json.load(open(os.path.join(dump, "meta.json")))
    t = L("node_type")
    left, right, leaf, nch = L("node_left"), L("node_right"), L("node_leaf"), L("node_nchildren")
    Nn = len(t)
    lf = np.zeros(Nn, np.int64)
    for i in range(Nn):
        lf[i] = leaf[i] if (t[i] & 1) else lf[left[i]]
    ls, le = L("node_link_start"), L("node_link_end")
    assert np.all(ls[1:] == le[:-1]) and ls[0] == 0
    link_ptr = np.concatenate([ls.astype(np.int64), le[-1:].astype(np.int64)])
    conds = meta["conductors"]
    cleaf = np.array([c["leaf_panels"] for c in conds], np.int64)
    surf, sptr = [], [0]
    for c in conds:
        surf += c["surf_outperm"]
        sptr.append(len(surf))
    out = {
        "node_type": t, "node_left": left, "node_right": right, "node_leaf_first": lf, "node_leaf_count": nch,
        "node_vertices": L("node_vertices"), "node_centroid": L("node_centroid"), "node_normal": L("node_normal"),
        "node_area": L("node_area"), "node_maxside": L("node_maxside"), "link_ptr": link_ptr,
        "link_src": L("link_src"), "leaf_diel": L("leaf_diel"),
        "cond_is_diel": np.array([1 if c["is_diel"] else 0 for c in conds], np.uint8),
        "cond_leaf_first": np.concatenate([[0], np.cumsum(cleaf)[:-1]]).astype(np.int64),
        "cond_leaf_count": cleaf,
        "cond_outperm": np.array([c["outperm"] for c in conds], np.float64),
        "cond_inperm": np.array([c["inperm"] for c in conds], np.float64),
        "cond_surf_ptr": np.array(sptr, np.int32),
        "cond_surf_outperm": np.array(surf if surf else [0.0], np.float64),
        "cond_names": np.array([c["name"] for c in conds]),
        "ref_link_coef": L("link_coef"), "ref_self_coef": L("self_coef"),
        "ref_mv_q": L("mv_q"), "ref_mv_v": L("mv_v"), "ref_cap": L("cap"),
        "ref_iterations": np.array(meta["gmres_iterations"], np.int32),
        "ref_counts": np.array([meta["panels"], meta["nodes"], meta["links"]], np.int64),
        "ref_max_mesh_eps": np.array(meta["max_mesh_eps"]),
        "ref_max_level": np.array(meta["max_level"]),
    }
    if os.path.exists(os.path.join(dump, "sup_nodes.npy")):
        out.update({"ref_sup_nodes": L("sup_nodes"), "ref_sup_index": L("sup_index"), "ref_sup_area": L("sup_area"),
                    "ref_sup_minv": L("sup_minv")})
    return out


# cases at the sizes the benchmark configurations name, too large to commit in
# full: the fixture keeps the counts, a SHA-256 of every model array in the C-ABI
# layout, the self coefficients, every PIN_STRIDE-th link coefficient, one
# seeded product, the GMRES iteration counts and the capacitance matrix
PIN_CASES = {
    # 2x2 crossing of 1x1x10 um bars at 3 um pitch, layers 1 um apart, vacuum;
    # -m0.0018 gives 5,088 panels (the "about 5k panels" configuration)
    "pin_crossing2x2_5k": (lambda: geo.crossing_2x2().text(), ["-m0.0018", "-t1e-4", "-pj", "-f0"]),
    # sphere R = 1 m, icosahedron subdivided 5 times (20,480 triangles), mesh
    # refinement off, link tolerance 1e-3
    "pin_sphere_20480": (lambda: geo.sphere_text(5), ["-m1e30", "-d1e-33", "-t1e-4", "-pj", "-f0"]),
}
PIN_STRIDE = 97
MODEL_KEYS = ("node_type", "node_left", "node_right", "node_leaf_first", "node_leaf_count", "node_vertices",
              "node_centroid", "node_normal", "node_area", "node_maxside", "link_ptr", "link_src", "leaf_diel",
              "cond_is_diel", "cond_leaf_first", "cond_leaf_count", "cond_outperm", "cond_inperm", "cond_surf_ptr",
              "cond_surf_outperm")


def array_sha256(a) -> str:
    """SHA-256 of an array's dtype, shape and little-endian bytes (C order)."""
    import hashlib
    a = np.ascontiguousarray(a)
    h = hashlib.sha256()
    h.update(("%s|%s|" % (a.dtype.newbyteorder("<").str, ",".join(str(x) for x in a.shape))).encode())
    h.update(a.astype(a.dtype.newbyteorder("<"), copy=False).tobytes())
    return h.hexdigest()


def compact(full: dict) -> dict:
    out = {"model_sha256": np.array(["%s:%s" % (k, array_sha256(full[k])) for k in MODEL_KEYS])}
    for k in ("cond_names", "ref_self_coef", "ref_mv_q", "ref_mv_v", "ref_cap", "ref_iterations", "ref_counts",
              "ref_max_mesh_eps", "ref_max_level", "cond_is_diel"):
        out[k] = full[k]
    idx = np.arange(0, len(full["ref_link_coef"]), PIN_STRIDE, dtype=np.int64)
    out["ref_link_coef_index"] = idx
    out["ref_link_coef_sample"] = full["ref_link_coef"][idx]
    return out


def main_pin(ref_dir: str = "", only=()):
    make_reference(ref_dir)
    dump_bin = os.path.join(ROOT, "oracle", "_ref", "fcref_dump")
    with tempfile.TemporaryDirectory() as tmp:
        for name, (text_fn, switches) in PIN_CASES.items():
            if only and name not in only:
                continue
            text = text_fn()
            inp = os.path.join(tmp, name + ".txt")
            with open(inp, "w") as f:
                f.write(text)
            dump = os.path.join(tmp, name + "_dump")
            subprocess.run([dump_bin, dump, inp] + switches + ["--mv", "1"], check=True,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            out = compact(convert(dump))
            out["switches"] = np.array(switches)
            import hashlib
            out["input_sha256"] = np.array(hashlib.sha256(text.encode()).hexdigest())
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
            print("%-22s panels %6d nodes %6d links %8d iterations %s" % (
                (name,) + tuple(out["ref_counts"]) + (list(out["ref_iterations"]),)))


# automatic refinement runs of the reference console (-a<err>): per-iteration
# panel and link counts and the final capacitance matrix, parsed from its report
AUTO_CASES = {
    "auto_crossing2x2": (lambda: geo.crossing_2x2().text(), ["-a0.01", "-f0"]),
    "auto_crossing2x2_slab": (lambda: geo.Crossing(k=2, length=10.0, pitch=3.0, gap=1.0, eps_r=3.9,
                                                   slab=(3.5, 1.0, 3.9, 15.0), name="c2slab").text(), ["-a0.02", "-f0"]),
}


def parse_report(text: str) -> dict:
    """Per-iteration panels/links and the last capacitance matrix of a console report."""
    panels, links, caps, cur = [], [], [], None
    lines = text.splitlines()
    for i, ln in enumerate(lines):
        if ln.startswith("Number of panels after refinement:") and (i + 1 < len(lines)) and \
                lines[i + 1].startswith("Number of links to be computed:"):
            panels.append(int(ln.split(":")[1]))
            links.append(int(lines[i + 1].split(":")[1]))
        if ln.startswith("Dimension "):
            n = int(ln.split()[1])
            cur = [[float(x) for x in lines[i + 1 + r].split()[1:1 + n]] for r in range(n)]
            caps.append(cur)
    return {"ref_auto_panels": np.array(panels, np.int64), "ref_auto_links": np.array(links, np.int64),
            "ref_cap": np.array(caps[-1]), "ref_auto_iterations": np.array(len(caps))}


def make_reference(ref_dir: str = ""):
    """Build oracle/_ref from the reference tree: ref_dir, else FCG_REFERENCE_DIR,
    else the default location oracle/Makefile names."""
    ref = ref_dir or os.environ.get("FCG_REFERENCE_DIR", "")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "-j8"] + (["REF=" + ref] if ref else []),
                   check=True)


def main_auto(ref_dir: str, only=()):
    make_reference(ref_dir)
    console = os.path.join(ROOT, "oracle", "_ref", "fcref")
    with tempfile.TemporaryDirectory() as tmp:
        for name, (text_fn, switches) in AUTO_CASES.items():
            if only and name not in only:
                continue
            text = text_fn()
            inp = os.path.join(tmp, name + ".txt")
            with open(inp, "w") as f:
                f.write(text)
            rep = subprocess.run([console, inp] + switches, check=True, capture_output=True, text=True).stdout
            out = parse_report(rep)
            out["input_text"] = np.frombuffer(text.encode(), np.uint8)
            out["switches"] = np.array(switches)
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
            print("%-22s iterations %d, panels %s" % (name, int(out["ref_auto_iterations"]), list(out["ref_auto_panels"])))


# -o / -c runs of the reference console: every list and panel file it
# writes (names relative to the input's directory), with the input saved as
# <name>.txt, since the file names and contents derive from it
OUTPUT_CASES = {
    "out_c22": (lambda: geo.crossing_2x2().text(), ["-m0.05", "-f0"]),
    "out_slab": (lambda: geo.Crossing(k=2, length=10.0, pitch=3.0, gap=1.0, eps_r=3.9,
                                      slab=(3.5, 1.0, 3.9, 15.0), name="c2slab").text(), ["-m0.05", "-f0"]),
}


def main_output(ref_dir: str, only=()):
    make_reference(ref_dir)
    console = os.path.join(ROOT, "oracle", "_ref", "fcref")
    for name, (text_fn, switches) in OUTPUT_CASES.items():
        if only and name not in only:
            continue
        with tempfile.TemporaryDirectory() as tmp:
            text = text_fn()
            inp = os.path.join(tmp, name + ".txt")
            with open(inp, "w") as f:
                f.write(text)
            subprocess.run([console, inp] + switches + ["-o", "-c"], check=True, capture_output=True, text=True)
            files = sorted(f for f in os.listdir(tmp) if f != name + ".txt")
            blob = {f: open(os.path.join(tmp, f)).read() for f in files}
        out = {"input_text": np.frombuffer(text.encode(), np.uint8), "switches": np.array(switches),
               "files_json": np.frombuffer(json.dumps(blob).encode(), np.uint8)}
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print("%-22s %d files" % (name, len(files)))


def main(ref_dir: str = "", *only):
    make_reference(ref_dir)
    dump_bin = os.path.join(ROOT, "oracle", "_ref", "fcref_dump")
    with tempfile.TemporaryDirectory() as tmp:
        for name, (text_fn, switches) in CASES.items():
            if only and name not in only:
                continue
            text = text_fn()
            inp = os.path.join(tmp, name + ".txt")
            with open(inp, "w") as f:
                f.write(text)
            dump = os.path.join(tmp, name + "_dump")
            subprocess.run([dump_bin, dump, inp] + switches + ["--mv", "2"], check=True,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            out = convert(dump)
            out["input_text"] = np.frombuffer(text.encode(), np.uint8)
            out["switches"] = np.array(switches)
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
            print("%-22s panels %6d nodes %6d links %8d" % ((name,) + tuple(out["ref_counts"])))


if __name__ == "__main__":
    args = sys.argv[1:]
    if args[1:] and all(a.startswith("pin_") for a in args[1:]):
        main_pin(args[0], args[1:])
    elif args[1:] and all(a.startswith("auto_") for a in args[1:]):
        main_auto(args[0], args[1:])
    elif args[1:] and all(a.startswith("out_") for a in args[1:]):
        main_output(args[0], args[1:])
    else:
        main(*args)
