"""The device near-field fill evaluates the analytic triangle potential in a
reduced-cost form (one atan2 per edge instead of two atan and two
divisions, guards without divisions). It must agree with the
reference-order formula to 1e-12 relative (of the larger of the value and
the triangle's 1/size scale) where the fill uses it, field points within
about a triangle size (the near band): random points, points in the plane
(coplanar neighbours), just above it, near edges and vertices, and on the
band edge. (Far away both forms lose accuracy to cancellation alike; the
fill uses quadrature there.)

The mixed-precision fill evaluates the same potential in FP32 in the source
triangle's scaled frame (fcg_potential32). Where it decides the reference's
guards itself it must agree with the FP64 formula to 5e-5 of the same scale;
it must decide every generic, in-plane, just-above-plane and band-edge point,
and it hands points where an R + l guard is too close to call in FP32 (near
a vertex, close to an edge itself) to the FP64 formula.
"""

import ctypes as C
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("pot") / "libpotcheck.so")
    subprocess.check_call(["g++", "-O2", "-shared", "-fPIC", "-ffp-contract=off",
                           os.path.join(HERE, "native", "potential_check.cpp"), "-o", out])
    L = C.CDLL(out)
    L.pot_pair.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.pot_pair.restype = None
    L.pot32_pair.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.pot32_pair.restype = None
    return L


def run(lib, tri, pts):
    tri = np.ascontiguousarray(tri, np.float32)
    pts = np.ascontiguousarray(pts, np.float64)
    n = len(tri)
    ref, fast = np.empty(n), np.empty(n)
    lib.pot_pair(n, tri.ctypes.data, pts.ctypes.data, ref.ctypes.data, fast.ctypes.data)
    return ref, fast


def cases(seed, n=20000, with_kind=False):
    rng = np.random.default_rng(seed)
    tri = rng.uniform(-1, 1, (n, 3, 3)) * rng.uniform(1e-6, 1e2, (n, 1, 1))
    cen = tri.mean(axis=1)
    size = np.linalg.norm(tri[:, 1] - tri[:, 0], axis=1)[:, None]
    nrm = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    nrm /= np.linalg.norm(nrm, axis=1)[:, None]
    kind = rng.integers(0, 6, n)
    off = rng.normal(size=(n, 3))
    pts = cen + size * off * 0.5                                    # generic, near
    a, b = rng.uniform(0, 1, (2, n, 1))
    inplane = tri[:, 0] + a * (tri[:, 1] - tri[:, 0]) + b * (tri[:, 2] - tri[:, 0])
    pts = np.where((kind == 1)[:, None], inplane * 1.5 - cen * 0.5, pts)                        # in the plane
    pts = np.where((kind == 2)[:, None], inplane + nrm * size * 1e-7, pts)                      # just above it
    edge = tri[:, 0] + a * (tri[:, 1] - tri[:, 0])
    pts = np.where((kind == 3)[:, None], edge + nrm * size * rng.uniform(-1e-4, 1e-4, (n, 1)), pts)  # near an edge
    pts = np.where((kind == 4)[:, None], tri[:, 2] + size * 1e-5 * off, pts)                    # near a vertex
    unit = off / np.linalg.norm(off, axis=1)[:, None]
    pts = np.where((kind == 5)[:, None], cen + size * unit, pts)                                # at the band edge
    if with_kind:
        return tri.astype(np.float32), pts, kind
    return tri.astype(np.float32), pts


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_fast_form_matches_reference_order(lib, seed):
    tri, pts = cases(seed)
    ref, fast = run(lib, tri, pts)
    assert np.all(np.isfinite(ref)) and np.all(np.isfinite(fast))
    size = np.linalg.norm(tri[:, 1].astype(np.float64) - tri[:, 0], axis=1)
    scale = np.maximum(np.abs(ref), 1.0 / size)
    err = np.abs(fast - ref) / scale
    assert err.max() < 1e-12, (err.max(), np.argmax(err))


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_fp32_form(lib, seed):
    tri, pts, kind = cases(seed, with_kind=True)
    tri = np.ascontiguousarray(tri, np.float32)
    pts = np.ascontiguousarray(pts, np.float32)
    n = len(tri)
    ref, f32, ok = np.empty(n), np.empty(n), np.empty(n, np.int32)
    lib.pot32_pair(n, tri.ctypes.data, pts.ctypes.data, ref.ctypes.data, f32.ctypes.data, ok.ctypes.data)
    size = np.linalg.norm(tri[:, 1].astype(np.float64) - tri[:, 0], axis=1)
    scale = np.maximum(np.abs(ref), 1.0 / size)
    decided = ok == 1
    err = np.abs(f32 - ref) / scale
    assert np.all(np.isfinite(f32[decided]))
    assert err[decided].max() < 5e-5, (err[decided].max(), np.argmax(np.where(decided, err, 0)))
    generic = np.isin(kind, [0, 1, 2, 5])
    assert decided[generic].all()
