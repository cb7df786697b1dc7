"""Panel coordinates as the reference's reader converts them: sscanf's "%f",
which rounds the decimal text to the nearest float exactly as the C
library's strtof does. The builder converts plain decimal tokens itself and
hands every other form to sscanf; both must give strtof's float for every
token. Without mesh refinement the model's leaves are the input triangles,
vertices in input order, so their coordinates are compared bit for bit with
libc strtof of the same text. No GPU."""

import ctypes
import ctypes.util
from decimal import Decimal, getcontext

import numpy as np
import pytest

import fastercap_gb300 as fc

getcontext().prec = 60
_libc = ctypes.CDLL(ctypes.util.find_library("c"))
_libc.strtof.restype = ctypes.c_float
_libc.strtof.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_char_p)]


def strtof(text):
    return np.float32(_libc.strtof(text.encode(), None))


def plain_forms(rng, value):
    """Decimal spellings of one value: %g, many digits, exponent, sign, bare point."""
    forms = ["%.9g" % value, "%.25f" % value, "%.17e" % value, "%.3E" % value]
    if value >= 0:
        forms.append("+%.12g" % value)
    if float(int(value)) == value:
        forms.append("%d." % int(value))
    s = "%.9f" % value
    if s.startswith("0."):
        forms.append(s[1:])  # ".123"
    return forms[int(rng.integers(len(forms)))]


# 240 panels: the reader converts lines as it parses them; 20,500: files of
# 20,000 lines and more are converted on all host threads before the parse
@pytest.mark.parametrize("seed,n_panels", [(0, 240), (1, 240), (2, 20500)])
def test_panel_coordinates_match_strtof(tmp_path, seed, n_panels):
    rng = np.random.default_rng(seed)
    rows, expect = [], []
    for i in range(n_panels):
        x0, y0 = rng.uniform(-5, 5, 2)
        a, b = rng.uniform(0.5, 2.0, 2)
        z = 3.0 * i  # panels far apart, one plane each
        coords = [x0, y0, z, x0 + a, y0, z, x0, y0 + b, z]
        toks = [plain_forms(rng, float(v)) for v in coords]
        sep = "\t" if i % 7 == 0 else " "
        rows.append("T c " + sep.join(toks))
        expect.append([strtof(t) for t in toks])
    # just off the midpoint between two floats: a conversion through double
    # lands on the midpoint and rounds to even, the wrong side in both cases
    for k, (base, sign) in enumerate(((Decimal(1), 1), (Decimal(1) + Decimal(2) ** -23, -1))):
        t = str(base + Decimal(2) ** -24 + sign * Decimal(2) ** -60)
        z = "%d" % (3 * n_panels + 700 + 3 * k)
        toks = (t, "0", z, "3", "0", z, "0", "1", z)
        assert np.float32(float(t)) != strtof(t)  # the case needs correct rounding
        rows.append("T c " + " ".join(toks))
        expect.append([strtof(x) for x in toks])
    # forms the builder leaves to sscanf: hexadecimal, a value below the float
    # range, an exponent glued to a sign, upper-case infix
    zs = ["%d" % (3 * n_panels + 600 + 3 * k) for k in range(3)]
    odd = [("0x1p-1", "0", zs[0], "1", "0", zs[0], "0", "1", zs[0]),
           ("1e-50", "0", zs[1], "1", "0", zs[1], "0", "1", zs[1]),
           ("0", "0", zs[2], "0X1.8P1", "0", zs[2], "0", "1", zs[2])]
    for toks in odd:
        rows.append("T c " + " ".join(toks))
        expect.append([strtof(t) for t in toks])
    path = tmp_path / "numbers.txt"
    path.write_text("0 number forms\n" + "\n".join(rows) + "\n")
    m = fc.Model.build(str(path), mesh_eps=1e30)
    a = m.arrays
    leaves = a["node_leaf_count"] == 1
    got = np.asarray(a["node_vertices"], np.float32).reshape(-1, 9)[leaves]
    want = np.array(expect, np.float32)
    assert got.shape == want.shape

    def rows_sorted(x):
        return x[np.lexsort(x.T[::-1])]
    np.testing.assert_array_equal(rows_sorted(got).view(np.uint32), rows_sorted(want).view(np.uint32))


def test_crlf_and_tabs_build_the_same_model(tmp_path):
    """Windows line ends and tab separators are whitespace to the reader, as
    to sscanf: the same panels with LF, CRLF and tab-separated lines build
    the same model, array for array."""
    rng = np.random.default_rng(7)
    lines = ["0 line ends"]
    for i in range(60):
        x0, y0 = rng.uniform(-5, 5, 2)
        v = [x0, y0, 3.0 * i, x0 + 1.5, y0, 3.0 * i, x0, y0 + 1.25, 3.0 * i]
        lines.append("T c%d " % (i % 3) + " ".join("%.9g" % t for t in v))
    models = []
    for name, text in (("lf", "\n".join(lines) + "\n"), ("crlf", "\r\n".join(lines) + "\r\n"),
                       ("tabs", "\n".join(l.replace(" ", "\t") for l in lines) + "\n")):
        path = tmp_path / (name + ".txt")
        path.write_bytes(text.encode())
        models.append(fc.Model.build(str(path), mesh_eps=0.2))
    ref = models[0]
    for m in models[1:]:
        assert list(m.names) == list(ref.names)
        for k, a in ref.arrays.items():
            np.testing.assert_array_equal(np.asarray(m.arrays[k]), np.asarray(a), err_msg=k)
