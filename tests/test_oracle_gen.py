"""The oracle's own workload generator (oracle/acg_oracle_gen.c) makes the
same graphs, byte for byte, as the product's generators (include/acg_io.h),
so that the CPU baseline and the reference arm of the benchmark can build their
inputs without loading the product library.  CPU only."""
import numpy as np
import pytest

from application_classification_gb300 import graph
from oracle import oracle


def _same(a, b):
    for f in ("node_feats", "edge_feats", "srcs", "dsts"):
        x, y = np.asarray(getattr(a, f)), np.asarray(getattr(b, f))
        assert x.shape == y.shape, f
        assert x.tobytes() == y.tobytes(), f


@pytest.mark.parametrize("name", ["er1k", "rmat12", "rmat10_6_9", "rmat13_10_20", "rmat11_40_60"])
def test_workloads_byte_equal(name):
    d0, p0, t0 = graph.workload(name)
    d1, p1, t1 = oracle.workload(name)
    _same(d0, d1)
    _same(p0, p1)
    assert np.array_equal(np.asarray(t0), t1)


def test_generators_byte_equal():
    _same(graph.gen_er(300, 2000, kv=5, ke=3, seed=7), oracle.gen_er(300, 2000, kv=5, ke=3, seed=7))
    _same(graph.gen_rmat(9, 8, kv=4, ke=6, seed=5), oracle.gen_rmat(9, 8, kv=4, ke=6, seed=5))
    # a sparse graph: planting needs new vertices and new edges
    g0 = graph.gen_er(50, 10, kv=3, ke=2, seed=3)
    g1 = oracle.gen_er(50, 10, kv=3, ke=2, seed=3)
    a = graph.plant(g0, 12, 30, 0.1, seed=9)
    b = oracle.plant(g1, 12, 30, 0.1, seed=9)
    _same(a[0], b[0])
    _same(a[1], b[1])
    assert np.array_equal(np.asarray(a[2]), b[2]) and np.array_equal(np.asarray(a[3]), b[3])
    _same(graph.fill_edges(a[0], a[0].num_edges + 40, seed=2), oracle.fill_edges(b[0], b[0].num_edges + 40, seed=2))
