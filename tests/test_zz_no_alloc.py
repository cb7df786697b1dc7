"""The no-allocation matrix-vector product (fcg_problem_matvec_device_noalloc).

Callers that cannot allocate device memory when they multiply - hosts that
reserve all device memory at start-up, hosts whose device memory belongs to
another allocator - use this entry point.
It must give the same result as fcg_problem_matvec_device (same kernels, so
the FP64 tolerance 1e-13 relative norm and the mixed 2e-6 both hold with
room), call after call, and refuse models too large for its fixed 32 MiB
scratch with a status instead of faulting. Device buffers for the inputs and
outputs come from the test (torch), not from the entry point.

This file sorts last so that a run stopping at its first failure has run
every other test before it.
"""

import numpy as np
import pytest

import fastercap_gb300 as fc
from conftest import load_golden, model_arrays

pytestmark = pytest.mark.gpu


def rel_norm(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("case", ["crossing2x2_m02", "random3", "crossing2x2_slab"])
@pytest.mark.parametrize("precision,tol", [(fc.PREC_FP64, 1e-13), (fc.PREC_MIXED, 2e-6)])
@pytest.mark.parametrize("k", [1, 3])
def test_noalloc_matches_allocating_matvec(case, precision, tol, k):
    torch = pytest.importorskip("torch")
    g = load_golden(case)
    with fc.Context(0) as ctx:
        p = ctx.problem(fc.Model.from_arrays(model_arrays(g)), precision)
        p.fill()
        n = p.n_panels
        q = torch.tensor(np.random.default_rng(11).uniform(-1, 1, (k, n)), dtype=torch.float64, device="cuda")
        v_ref = torch.empty_like(q)
        torch.cuda.synchronize()  # the library works on its own stream
        p.matvec_device(q.data_ptr(), v_ref.data_ptr(), k)
        outs = []
        for _ in range(2):  # two calls in a row share (and reuse) the scratch
            v = torch.full_like(q, float("nan"))
            torch.cuda.synchronize()
            code = p.matvec_device_noalloc(q.data_ptr(), v.data_ptr(), k)
            assert code == fc.NORMAL_END, fc.last_error()
            outs.append(v.cpu().numpy())
        ref = v_ref.cpu().numpy()
        for o in outs:
            assert rel_norm(o, ref) < tol
        assert rel_norm(outs[1], outs[0]) < tol
        p.close()


@pytest.mark.parametrize("precision,tol", [(fc.PREC_FP64, 1e-13), (fc.PREC_MIXED, 2e-6)])
def test_noalloc_records_into_a_cuda_graph(precision, tol):
    """Called while the caller records a CUDA graph on the problem's own
    (caller-owned) stream, the product goes into the graph; every replay
    computes the product of what the input buffer then holds, equal to
    fcg_problem_matvec_device's."""
    torch = pytest.importorskip("torch")
    g = load_golden("crossing2x2_m02")
    k = 3
    with fc.Context(0) as ctx:
        s = torch.cuda.Stream()
        p = ctx.problem(fc.Model.from_arrays(model_arrays(g)), precision, stream=s.cuda_stream)
        p.fill()
        n = p.n_panels
        q = torch.tensor(np.random.default_rng(5).uniform(-1, 1, (k, n)), dtype=torch.float64, device="cuda")
        v = torch.zeros_like(q)
        torch.cuda.synchronize()
        # one call before the first recording resolves the scratch address
        assert p.matvec_device_noalloc(q.data_ptr(), v.data_ptr(), k) == fc.NORMAL_END, fc.last_error()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=s):
            code = p.matvec_device_noalloc(q.data_ptr(), v.data_ptr(), k)
        assert code == fc.NORMAL_END, fc.last_error()
        ref = torch.empty_like(q)
        for seed in (6, 7):
            q.copy_(torch.from_numpy(np.random.default_rng(seed).uniform(-1, 1, (k, n))))
            v.fill_(float("nan"))
            torch.cuda.synchronize()
            graph.replay()
            torch.cuda.synchronize()
            p.matvec_device(q.data_ptr(), ref.data_ptr(), k)
            assert rel_norm(v.cpu().numpy(), ref.cpu().numpy()) < tol
        p.close()


def test_noalloc_rejects_models_beyond_its_scratch(tmp_path):
    torch = pytest.importorskip("torch")
    from fastercap_gb300 import geometry as geo
    path = tmp_path / "sphere.txt"
    geo.write_sphere(str(path), 6)  # 163,839 nodes
    m = fc.Model.build(str(path), mesh_eps=1e30, eps_ratio=1e-32)
    # 8 right-hand sides, mixed: 3 double + 1 float arrays of nodes x 8 values
    # = 163,839 x 8 x 28 bytes = 36.7 MB, above the 32 MiB scratch
    need = m.n_nodes * 8 * (3 * 8 + 4)
    assert need > (32 << 20), "the case no longer exceeds the scratch; pick a larger model"

    with fc.Context(0) as ctx:
        p = ctx.problem(m, fc.PREC_MIXED)
        p.fill()
        q = torch.zeros((8, p.n_panels), dtype=torch.float64, device="cuda")
        v = torch.zeros_like(q)
        torch.cuda.synchronize()
        code = p.matvec_device_noalloc(q.data_ptr(), v.data_ptr(), 8)
        assert code == fc.OUT_OF_MEMORY
        assert "32" in fc.last_error() or "scratch" in fc.last_error()
        # within the limit the same problem works
        q1 = torch.tensor(np.random.default_rng(2).uniform(-1, 1, (1, p.n_panels)), dtype=torch.float64, device="cuda")
        v1 = torch.empty_like(q1)
        v2 = torch.empty_like(q1)
        torch.cuda.synchronize()
        assert p.matvec_device_noalloc(q1.data_ptr(), v1.data_ptr(), 1) == fc.NORMAL_END
        p.matvec_device(q1.data_ptr(), v2.data_ptr(), 1)
        assert rel_norm(v1.cpu().numpy(), v2.cpu().numpy()) < 2e-6
        p.close()
