"""Build the in-tree native libraries.

* ``fastercap_gb300/libfastercap_gb300.so`` — the product: sm_103a CUDA kernels
  (``csrc/problem.cu``), the host model builder and the C ABI (``host/*.cpp``).
* ``fastercap_gb300/fastercap_gb300`` — headless console with the reference's
  command line.
* ``oracle/liboracle.so`` — the CPU oracle used by the tests and the CPU
  baseline of the benchmark (test infrastructure, never loaded by the product).
* ``oracle/_ref/`` — the reference solver itself, only where its source tree
  is present (``make -C oracle``).

Host C/C++ is compiled with ``-ffp-contract=off`` so that the model builder
makes the same floating-point decisions on x86-64 and AArch64.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CXXFLAGS = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-Wall", "-Wno-unused-function"]
# reference source tree for the oracle build: FCG_REFERENCE_DIR, else the
# default location named by oracle/Makefile (the recipe that reads it)
REFERENCE = os.environ.get("FCG_REFERENCE_DIR")
# per-file device flags: the link construction, the mesh refinement and the
# super hierarchy round every operation like the host builder (no fused
# multiply-add), so both take the same decisions and make the same elements
CU_FLAGS = {"link_build.cu": ["-fmad=false"], "mesh_build.cu": ["-fmad=false"], "super_build.cu": ["-fmad=false"]}

LIB = os.path.join(HERE, "libfastercap_gb300.so")
CLI = os.path.join(HERE, "fastercap_gb300")
ORACLE_LIB = os.path.join(ROOT, "oracle", "liboracle.so")


def _run_all(cmds):
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)) for c in cmds]
    failed = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((c, out))
        elif out and out.strip():
            sys.stderr.write(out)
    if failed:
        msg = "\n".join("$ %s\n%s" % (" ".join(c), o) for c, o in failed)
        raise RuntimeError("native build failed:\n" + msg)


def _newer(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build(verbose: bool = False, reference: bool = True) -> None:
    os.makedirs(BUILD, exist_ok=True)
    csrc = os.path.join(HERE, "csrc")
    host = os.path.join(HERE, "host")
    headers = [os.path.join(csrc, f) for f in os.listdir(csrc) if f.endswith((".h", ".hpp", ".cuh"))]
    headers += [os.path.join(host, f) for f in os.listdir(host) if f.endswith((".h", ".hpp"))]
    headers.append(os.path.join(ROOT, "include", "fastercap_gb300.h"))
    cu = [os.path.join(csrc, f) for f in sorted(os.listdir(csrc)) if f.endswith(".cu")]
    cpp = [os.path.join(host, f) for f in ("model_builder.cpp", "api.cpp", "server.cpp")]
    objs, cmds = [], []
    for src in cu:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if _newer(obj, [src] + headers):
            cmds.append([NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off"]
                        + CU_FLAGS.get(os.path.basename(src), []) + ["-c", src, "-o", obj])
    for src in cpp:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if _newer(obj, [src] + headers):
            cmds.append(["g++"] + CXXFLAGS + ["-I/usr/local/cuda/include", "-c", src, "-o", obj])
    oracle_src = os.path.join(ROOT, "oracle", "fcoracle.c")
    if os.path.exists(oracle_src) and _newer(ORACLE_LIB, [oracle_src, os.path.join(ROOT, "oracle", "fcoracle.h")]):
        cmds.append(["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-std=c11", "-Wall",
                     oracle_src, "-o", ORACLE_LIB, "-lm"])
    if cmds:
        _run_all(cmds)
    if _newer(LIB, objs):
        _run_all([[NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]])
    cli_src = os.path.join(host, "cli_main.cpp")
    if _newer(CLI, [cli_src, LIB]):
        _run_all([["g++", "-O2", "-std=c++17", cli_src, "-o", CLI, "-L" + HERE, "-lfastercap_gb300",
                   "-Wl,-rpath,$ORIGIN"]])
    if reference and shutil.which("make"):
        oracle_dir = os.path.join(ROOT, "oracle")
        ref = ["REF=" + REFERENCE] if REFERENCE else []
        have = subprocess.run(["make", "-s", "-C", oracle_dir, "have-ref"] + ref,
                              stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL).returncode == 0
        if have:
            _run_all([["make", "-s", "-C", oracle_dir, "-j8"] + ref])


if __name__ == "__main__":
    build(verbose=True)
