"""The Python binding's ctypes structures against the C header they mirror:
a C program compiled against include/fastercap_gb300.h prints every
structure's size and its members' offsets, and each must equal the ctypes
layout (a member added on one side only would shift every later field and
be read as garbage, with no error). No GPU."""

import os
import shutil
import subprocess

import pytest

import fastercap_gb300 as fc
from conftest import ROOT

STRUCTS = {
    "fcg_build_options": fc.BuildOptions,
    "fcg_model_arrays": fc.ModelArrays,
    "fcg_model_info": fc.ModelInfo,
    "fcg_problem_stats": fc.ProblemStats,
    "fcg_solve_options": fc.SolveOptions,
    "fcg_server_config": fc.ServerConfig,
    "fcg_job_info": fc.JobInfo,
    "fcg_server_stats": fc.ServerStats,
}


def c_layout(tmp_path):
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "fastercap_gb300.h"', "int main(void) {"]
    for cname, cls in STRUCTS.items():
        lines.append('    printf("%s sizeof %%zu\\n", sizeof(%s));' % (cname, cname))
        for field, _ in cls._fields_:
            lines.append('    printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, field, cname, field))
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True,
                   capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    layout = {}
    for line in out.splitlines():
        cname, key, value = line.split()
        layout[(cname, key)] = int(value)
    return layout


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs a C compiler")
def test_ctypes_structures_match_the_c_header(tmp_path):
    layout = c_layout(tmp_path)
    for cname, cls in STRUCTS.items():
        assert layout[(cname, "sizeof")] == fc.C.sizeof(cls), cname
        for field, _ in cls._fields_:
            assert layout[(cname, field)] == getattr(cls, field).offset, (cname, field)


def test_solve_options_defaults_are_the_reference_defaults():
    """A zero-initialised fcg_solve_options (what a C host's aggregate
    initialiser leaves for members it does not name) means: the reference's
    iteration cap, measured right-hand-side width, default two-level size and
    refinement, and the FP32-pair Krylov basis."""
    o = fc.SolveOptions()
    assert (o.max_iter, o.rhs_width, o.precond_dim, o.refine, o.krylov) == (0, 0, 0, 0, fc.KRYLOV_PAIR)
    assert fc.KRYLOV_PAIR == 0 and fc.KRYLOV_FP64 == 1
