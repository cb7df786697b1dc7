import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

GOLDEN = os.path.join(ROOT, "tests", "golden")
MODEL_KEYS = ["node_type", "node_left", "node_right", "node_leaf_first", "node_leaf_count", "node_vertices",
              "node_centroid", "node_normal", "node_area", "node_maxside", "link_ptr", "link_src", "leaf_diel",
              "cond_is_diel", "cond_leaf_first", "cond_leaf_count", "cond_outperm", "cond_inperm", "cond_surf_ptr",
              "cond_surf_outperm"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: longer CPU test")
    from fastercap_gb300 import build
    build.build(reference=False)


def golden_names():
    """cases with the reference's full model dump (auto_* are console-report
    fixtures, out_* the console's -o/-c files, pin_* compact fixtures of the
    benchmark-size cases)"""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if not os.path.basename(p).startswith(("auto_", "out_", "pin_")))


def load_golden(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: d[k] for k in d.files}


def model_arrays(g):
    return {k: g[k] for k in MODEL_KEYS}


def switch_value(switches, prefix, default):
    for s in switches:
        s = str(s)
        if s.startswith(prefix) and not (prefix == "-m" and s.startswith("-mc")):
            return float(s[len(prefix):])
    return default


def build_from_golden(g, tmp_path):
    """Run this library's model builder on the golden case's input."""
    import fastercap_gb300 as fc
    inp = tmp_path / "input.txt"
    inp.write_bytes(bytes(g["input_text"]))
    sw = [str(s) for s in g["switches"]]
    return fc.Model.build(str(inp), mesh_eps=switch_value(sw, "-m", 0.1), eps_ratio=switch_value(sw, "-d", 1.0))


def solve_params(g):
    """(GMRES tolerance, preconditioner: 0 none, 1 Jacobi, 2 two-level)"""
    sw = [str(s) for s in g["switches"]]
    tol = switch_value(sw, "-t", 0.01)
    precond = 0 if "-pn" in sw else (2 if any(s.startswith("-ps") for s in sw) else 1)
    return tol, precond


def super_dim(g):
    """the two-level preconditioner dimension of -ps<dim> (0 if absent)"""
    for s in g["switches"]:
        s = str(s)
        if s.startswith("-ps"):
            return int(s[3:])
    return 0


@pytest.fixture(params=golden_names())
def golden(request):
    return request.param, load_golden(request.param)
