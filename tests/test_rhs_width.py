"""Right-hand-side width of the batched solves.

With fcg_solve_options.rhs_width = 0 a mixed problem of at least 4M links
picks its width by measuring the link product at 4, 8, 16 columns and at all
conductors; the capacitance matrix does not depend on the width beyond the
mixed path's tolerance (every column is its own GMRES solve, whatever batch
it runs in), and the stats report the width used."""

import numpy as np
import pytest

import fastercap_gb300 as fc
from fastercap_gb300 import geometry as geo

pytestmark = pytest.mark.gpu


def test_measured_width_gives_the_same_matrix(tmp_path):
    path = tmp_path / "c6.txt"
    geo.Crossing(k=6, length=20.0, pitch=2.5, gap=1.5, name="c6").write(str(path))
    with fc.Context(0) as ctx:
        m = fc.Model.build(str(path), mesh_eps=1.5e-3, eps_ratio=1.0, ctx=ctx)  # 14,400 panels, 4.66M links
        assert m.n_links >= 4 << 20 and len(m.conductor_names) == 12
        caps = {}
        for width in (0, 12, 4, 1):
            p = ctx.problem(m, fc.PREC_MIXED)
            p.fill()
            caps[width], _ = p.solve(tol=1e-6, rhs_width=width)
            used = p.stats()["rhs_width"]
            p.close()
            if width == 0:
                assert used in (4, 8, 12)
            else:
                assert used == width
        for width in (12, 4, 1):
            err = np.abs(caps[0] - caps[width]) / np.abs(caps[width])
            assert err.max() < 1e-4, (width, err.max())
