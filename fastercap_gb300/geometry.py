"""Deterministic FastCap-format geometry generators for the benchmark workloads.

The files written here use FasterCap's single-file input format (a main
section of ``C``/``D`` statements, then ``File <name>`` sections holding the
``Q``/``T`` panels, as described in the reference's
``hlp/InputFile/InputFile_single_file.htm`` and ``hlp/InputFile/3D/*.htm``).

Conventions (fixed, so every consumer reads the same geometry):

* bus crossings are written in micrometres as plain numbers (the solver reads
  them as metres, so reported capacitances are 1e6 x the micrometre-scale
  values; both the reference and this library read the same file);
* each bar is a closed box of six ``Q`` faces whose corners are ordered so the
  Newell normal points out of the box;
* a ``k x k`` crossing has ``k`` bars along x in the lower layer (z in
  [0, h]) and ``k`` bars along y in the upper layer, ``gap`` above it
  (edge-to-edge), ``pitch`` centre-to-centre, centred on the origin;
* spheres are icosahedra subdivided ``depth`` times (20 * 4**depth triangles),
  vertices projected onto the sphere, written with ``%.9e``.
"""

from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np


def _newell(pts):
    n = np.zeros(3)
    m = len(pts)
    for i in range(m):
        a, b = np.asarray(pts[i], float), np.asarray(pts[(i + 1) % m], float)
        n[0] += (a[1] - b[1]) * (a[2] + b[2])
        n[1] += (a[2] - b[2]) * (a[0] + b[0])
        n[2] += (a[0] - b[0]) * (a[1] + b[1])
    return n


def box_faces(x0, y0, z0, x1, y1, z1):
    """Six quadrilaterals of an axis-aligned box, corners ordered outward."""
    faces = [
        [(x0, y0, z1), (x1, y0, z1), (x1, y1, z1), (x0, y1, z1)],  # +z
        [(x0, y0, z0), (x0, y1, z0), (x1, y1, z0), (x1, y0, z0)],  # -z
        [(x1, y0, z0), (x1, y1, z0), (x1, y1, z1), (x1, y0, z1)],  # +x
        [(x0, y0, z0), (x0, y0, z1), (x0, y1, z1), (x0, y1, z0)],  # -x
        [(x0, y1, z0), (x0, y1, z1), (x1, y1, z1), (x1, y1, z0)],  # +y
        [(x0, y0, z0), (x1, y0, z0), (x1, y0, z1), (x0, y0, z1)],  # -y
    ]
    centre = np.array([(x0 + x1) / 2, (y0 + y1) / 2, (z0 + z1) / 2])
    for f in faces:
        n = _newell(f)
        c = np.mean(np.asarray(f, float), axis=0)
        assert np.dot(n, c - centre) > 0, "box face is not outward"
    return faces


def _fmt(v):
    return "%.9g" % v


def _q_line(name, quad):
    return "Q %s  " % name + "  ".join(" ".join(_fmt(c) for c in p) for p in quad)


@dataclass
class Crossing:
    """A k x k bus crossing (all lengths in micrometres)."""

    k: int
    length: float
    pitch: float
    gap: float
    width: float = 1.0
    height: float = 1.0
    eps_r: float = 1.0
    # dielectric interface above the bars: (z, outperm above, inperm below,
    # half-extent in x and y); None for a homogeneous medium
    slab: tuple | None = None
    name: str = "crossing"
    meta: dict = field(default_factory=dict)

    def bars(self):
        """Yield (conductor name, box) for every bar, lower layer first."""
        h, w, L = self.height, self.width, self.length
        off = [(i - (self.k - 1) / 2.0) * self.pitch for i in range(self.k)]
        for i, yc in enumerate(off):
            yield "x%d" % (i + 1), (-L / 2, yc - w / 2, 0.0, L / 2, yc + w / 2, h)
        z0 = h + self.gap
        for i, xc in enumerate(off):
            yield "y%d" % (i + 1), (xc - w / 2, -L / 2, z0, xc + w / 2, L / 2, z0 + h)

    def text(self) -> str:
        out = ["* %s: %dx%d bus crossing, length %g pitch %g gap %g (um)" % (
            self.name, self.k, self.k, self.length, self.pitch, self.gap)]
        names = []
        for cname, _ in self.bars():
            names.append(cname)
            out.append("C %s.txt  %s  0.0 0.0 0.0" % (cname, _fmt(self.eps_r)))
        if self.slab is not None:
            z, eout, ein, half = self.slab
            out.append("D slab.txt  %s %s  0.0 0.0 0.0  0.0 0.0 %s" % (
                _fmt(eout), _fmt(ein), _fmt(z + 1.0)))
        out.append("End")
        for cname, box in self.bars():
            out.append("File %s.txt" % cname)
            out.append("* bar %s" % cname)
            for f in box_faces(*box):
                out.append(_q_line(cname, f))
            out.append("End")
        if self.slab is not None:
            z, eout, ein, half = self.slab
            out.append("File slab.txt")
            out.append("* planar dielectric interface at z = %s" % _fmt(z))
            quad = [(-half, -half, z), (half, -half, z), (half, half, z), (-half, half, z)]
            out.append(_q_line("slab", quad))
            out.append("End")
        return "\n".join(out) + "\n"

    def write(self, path: str) -> str:
        with open(path, "w") as f:
            f.write(self.text())
        return path


def crossing_2x2() -> Crossing:
    """2x2 crossing in vacuum: bars 1x1x10 um at 3 um pitch, layers at z=0 and z=2."""
    return Crossing(k=2, length=10.0, pitch=3.0, gap=1.0, name="crossing2x2")


def crossing_8x8_slab() -> Crossing:
    """8x8 crossing, bars 1x1x40 um at 2 um pitch, layers 1.5 um apart, in an
    eps_r=3.9 slab whose top interface (to eps_r=1) is the plane z=4 um,
    modelled as a square three times the crossing footprint."""
    return Crossing(k=8, length=40.0, pitch=2.0, gap=1.5, eps_r=3.9,
                    slab=(4.0, 1.0, 3.9, 60.0), name="crossing8x8_slab")


def crossing_batch(seed: int = 0, n: int = 32, kmin: int = 2, kmax: int = 10) -> list:
    """n random crossings drawn in order from one numpy default_rng(seed):
    per geometry k ~ U{kmin..kmax}, length ~ U[10, 60], pitch ~ U[2, 4],
    gap ~ U[1, 3] (um), vacuum (the uneven-batch workload: 32 crossings from
    seed 0)."""
    rng = np.random.default_rng(seed)
    out = []
    for g in range(n):
        k = int(rng.integers(kmin, kmax + 1))
        length = float(rng.uniform(10.0, 60.0))
        pitch = float(rng.uniform(2.0, 4.0))
        gap = float(rng.uniform(1.0, 3.0))
        out.append(Crossing(k=k, length=round(length, 6), pitch=round(pitch, 6), gap=round(gap, 6),
                            name="batch%d_%d" % (seed, g), meta={"seed": seed, "index": g}))
    return out


def random_crossing(seed: int, kmin: int = 2, kmax: int = 10) -> Crossing:
    """Random crossing drawn from numpy default_rng(seed), in this order:
    k ~ U{kmin..kmax}, length ~ U[10, 60], pitch ~ U[2, 4], gap ~ U[1, 3] (um),
    vacuum."""
    rng = np.random.default_rng(seed)
    k = int(rng.integers(kmin, kmax + 1))
    length = float(rng.uniform(10.0, 60.0))
    pitch = float(rng.uniform(2.0, 4.0))
    gap = float(rng.uniform(1.0, 3.0))
    return Crossing(k=k, length=round(length, 6), pitch=round(pitch, 6), gap=round(gap, 6),
                    name="random%d" % seed, meta={"seed": seed})


def icosphere(depth: int, radius: float = 1.0):
    """Vertices (V,3) and outward triangles (T,3) of a subdivided icosahedron."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t),
             (0, -1, -t), (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(v, float) / np.linalg.norm(v) for v in verts]
    tris = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
            (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
            (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(depth):
        cache = {}

        def mid(a, b):
            key = (a, b) if a < b else (b, a)
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nt = []
        for a, b, c in tris:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nt += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        tris = nt
    V = np.array(verts) * radius
    T = np.array(tris, dtype=np.int64)
    # orient every triangle outward (centroid direction)
    a, b, c = V[T[:, 0]], V[T[:, 1]], V[T[:, 2]]
    n = np.cross(b - a, c - a)
    flip = np.einsum("ij,ij->i", n, a + b + c) < 0
    T[flip] = T[flip][:, [0, 2, 1]]
    return V, T


def sphere_text(depth: int, radius: float = 1.0) -> str:
    V, T = icosphere(depth, radius)
    lines = ["* sphere radius %g, icosahedron subdivided %d times, %d triangles" % (radius, depth, len(T)),
             "C sphere.txt  1.0  0.0 0.0 0.0", "End", "File sphere.txt", "* sphere"]
    for a, b, c in T:
        lines.append("T sphere  %.9e %.9e %.9e  %.9e %.9e %.9e  %.9e %.9e %.9e" % (
            *V[a], *V[b], *V[c]))
    lines.append("End")
    return "\n".join(lines) + "\n"


def write_sphere(path: str, depth: int, radius: float = 1.0) -> str:
    with open(path, "w") as f:
        f.write(sphere_text(depth, radius))
    return path


def write_all(directory: str) -> dict:
    """Write the standard workloads into ``directory`` and return their paths."""
    os.makedirs(directory, exist_ok=True)
    out = {
        "crossing2x2": crossing_2x2().write(os.path.join(directory, "crossing2x2.txt")),
        "crossing8x8_slab": crossing_8x8_slab().write(os.path.join(directory, "crossing8x8_slab.txt")),
    }
    for d in (5, 6, 7):
        out["sphere%d" % (20 * 4 ** d)] = write_sphere(os.path.join(directory, "sphere_d%d.txt" % d), d)
    return out
