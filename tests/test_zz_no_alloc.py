"""acg_initial_mu_noalloc: the initial mu computed with no memory allocation.

Some callers cannot allocate device memory where they call the matcher: code
running while a stream is captured into a CUDA graph, serving loops held to a
fixed memory budget, hosts embedding the library behind another framework's
allocator.  This entry point keeps its scratch in a fixed file-scope device
array instead.  The test calls it through the C ABI twice in a row and checks
each result against the regular entry point (acg_match_graphs with zero BP
iterations, FP64), with the FP64 tolerance of the other parity tests.  It runs
last (file name) and passes alone in a fresh process as well.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import load_golden
from application_classification_gb300 import _lib, matcher

pytestmark = pytest.mark.gpu

FP64_REL = 1e-10


def _noalloc(dev_data, dev_pat, out, stream):
    L = _lib.lib()
    st = L.acg_initial_mu_noalloc(C.c_void_p(dev_data.node_feats.data_ptr()), dev_data.num_nodes,
                                  dev_data.node_feat_dim, C.c_void_p(dev_pat.node_feats.data_ptr()),
                                  dev_pat.num_nodes, C.c_void_p(out.data_ptr()),
                                  C.c_void_p(stream.cuda_stream))
    _lib.check(st, "acg_initial_mu_noalloc")


@pytest.mark.parametrize("name", ["er300", "georgiy", "rmat9"])
def test_noalloc_matches_regular_entry_point(cuda, name):
    import torch

    d, p, _ = load_golden(name)
    ref = matcher.match(d, p, "fp64", num_iters=0)  # regular path, allocates its workspaces
    dd, dp = matcher.DeviceGraph(d), matcher.DeviceGraph(p)
    stream = torch.cuda.current_stream()
    for _ in range(2):  # two calls in a row share the static scratch
        out = torch.full((d.num_nodes, p.num_nodes), float("nan"), dtype=torch.float64, device=cuda)
        _noalloc(dd, dp, out, stream)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.isfinite(got).all()
        assert np.abs(got - ref).max() <= FP64_REL * max(1.0, np.abs(ref).max())


def _numpy_mu0(x, y):
    """mu[r][p] = -d(r, p) - log sum_r' exp(-d(r', p)), d the Euclidean distance
    (the reference's initial MU, main.cu:109-120), in FP64 numpy."""
    d = np.sqrt(((x[:, None, :] - y[None, :, :]) ** 2).sum(-1))
    m = (-d).max(0)
    return -d - (m + np.log(np.exp(-d - m).sum(0)))


def test_noalloc_limits_and_stale_partials(cuda):
    """The largest pattern (128 vertices) and feature dimension (32): two rows
    per block, the statistics pass over 5,000 rows strides its grid several
    times and the output pass its 640,000 entries too.  The second call has a
    different, smaller input (fewer blocks than the first): a read of the first
    call's partials left in the shared array would change its result."""
    import torch

    rng = np.random.default_rng(7)
    stream = torch.cuda.current_stream()
    for n, p, k in ((5000, 128, 32), (300, 128, 32), (5000, 128, 32)):
        x = rng.normal(size=(n, k))
        y = rng.normal(size=(p, k))
        ref = _numpy_mu0(x, y)
        dx = matcher.DeviceGraph.from_tensors(torch.from_numpy(x).to(cuda), torch.zeros((0, 1)),
                                              torch.zeros(0), torch.zeros(0))
        dy = matcher.DeviceGraph.from_tensors(torch.from_numpy(y).to(cuda), torch.zeros((0, 1)),
                                              torch.zeros(0), torch.zeros(0))
        out = torch.full((n, p), float("nan"), dtype=torch.float64, device=cuda)
        _noalloc(dx, dy, out, stream)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.isfinite(got).all()
        assert np.abs(got - ref).max() <= FP64_REL * max(1.0, np.abs(ref).max())


def test_noalloc_rejects_oversized_pattern(cuda):
    import torch

    x = torch.zeros((4, 13), dtype=torch.float64, device=cuda)
    y = torch.zeros((129, 13), dtype=torch.float64, device=cuda)
    out = torch.zeros((4, 129), dtype=torch.float64, device=cuda)
    st = _lib.lib().acg_initial_mu_noalloc(C.c_void_p(x.data_ptr()), 4, 13, C.c_void_p(y.data_ptr()),
                                           129, C.c_void_p(out.data_ptr()), None)
    assert st == 5  # ACG_ERR_UNSUPPORTED
    assert b"129 pattern vertices" in _lib.lib().acg_last_error()
