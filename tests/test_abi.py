"""C ABI surface: the library loads and exports every declared entry point."""

import ctypes
import os
import re
import subprocess

import fastercap_gb300 as fc
from conftest import ROOT


def declared_functions():
    src = open(os.path.join(ROOT, "include", "fastercap_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fcg_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    L = fc.lib()
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", fc.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (fcg_[a-z0-9_]+)", out))
    assert set(names) <= exported


def test_no_torch_in_the_boundary():
    src = open(os.path.join(ROOT, "include", "fastercap_gb300.h")).read()
    assert "torch" not in src and "at::" not in src


def test_cli_usage_error():
    cli = os.path.join(ROOT, "fastercap_gb300", "fastercap_gb300")
    r = subprocess.run([cli, "-zz"], capture_output=True, text=True)
    assert r.returncode == fc.COMMAND_LINE_ERROR
    r = subprocess.run([cli, "in.txt", "-g"], capture_output=True, text=True)
    assert r.returncode == fc.COMMAND_LINE_ERROR


def test_cli_missing_input(tmp_path):
    cli = os.path.join(ROOT, "fastercap_gb300", "fastercap_gb300")
    r = subprocess.run([cli, str(tmp_path / "missing.txt")], capture_output=True, text=True)
    assert r.returncode == fc.CANNOT_OPEN_FILE
