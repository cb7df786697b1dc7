"""The integration glue a FasterCap maintainer adds,
compiled from oracle/integration_glue.cpp against the reference's own objects
(oracle/Makefile) and run on the reference's models: the arrays it flattens
from CMultHier pass fcg_model_arrays_check and equal, array by array, the
model this library's builder makes from the same input.

Needs oracle/_ref/fcref_glue, which builds only where the reference source
tree is present; elsewhere the test is skipped."""

import os
import subprocess

import numpy as np
import pytest

import fastercap_gb300 as fc
from conftest import MODEL_KEYS, ROOT, build_from_golden, load_golden

GLUE = os.path.join(ROOT, "oracle", "_ref", "fcref_glue")
CASES = ["crossing2x2_m05", "crossing2x2_slab", "merged_cubes", "random3", "sphere_d2"]


@pytest.mark.skipif(not os.path.exists(GLUE), reason="oracle/_ref/fcref_glue not built (no reference tree)")
@pytest.mark.parametrize("name", CASES)
def test_glue_flattens_the_reference_model_into_the_c_abi(name, tmp_path):
    g = load_golden(name)
    inp = tmp_path / "input.txt"
    inp.write_bytes(bytes(g["input_text"]))
    out = tmp_path / "glue"
    r = subprocess.run([GLUE, str(out), str(inp)] + [str(s) for s in g["switches"]], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    glue = {k: np.load(str(out / (k + ".npy"))) for k in MODEL_KEYS}
    m = build_from_golden(g, tmp_path)
    for k in MODEL_KEYS:
        a, b = np.asarray(m.arrays[k]), glue[k]
        if k == "cond_surf_outperm":
            a = a[: len(b)]
        np.testing.assert_array_equal(a.reshape(b.shape), b, err_msg=k)
    # the glue's arrays are accepted by the library as they are
    assert fc.Model.from_arrays(glue, list(m.names)).n_links == int(g["ref_counts"][2])

