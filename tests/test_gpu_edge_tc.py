"""The edge phase with the costs recomputed on the tensor cores (acg_edge_tc.cu)
against the edge phase that reads the stored edge cost matrix, and against the
oracle.

Both compute d(e, q) with the same arithmetic (the centred TF32-split cross
term, FP32 norms, the exact recompute of near pairs), so the maxima and with
them mu are the same bits; the oracle bound is the mixed path's 1e-4.  The
cases cover ragged last tiles, feature dims 1..24, 1..64 pattern edges, a hub
vertex whose in-edges span many chunks (partial rows merged by the CTA that
completes the vertex), vertices without in-edges, and repeated launches (the
chunk counters are left at zero).
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from oracle import oracle
from application_classification_gb300 import graph, matcher
from application_classification_gb300._lib import AcgError

pytestmark = pytest.mark.gpu

MIXED_ABS = 1e-4


def _both(d, p, **kw):
    data = matcher.DataGraph(d)
    out = {}
    for kern in ("fused", "stored"):
        plan = matcher.Plan(data, p, "mixed", edge_kernel=kern, **kw)
        a = plan.run().cpu().numpy()
        b = plan.run().cpu().numpy()  # the chunk counters were reset by the first launch
        plan.stats()  # raises if a device-side wait gave up
        assert np.array_equal(a, b), kern
        out[kern] = a
        plan.close()
    data.close()
    return out


@pytest.mark.parametrize("name", golden_names())
def test_fused_golden(cuda, name):
    d, p, ref = load_golden(name)
    if p.num_edges == 0 or d.num_edges == 0:
        pytest.skip("no edge phase")
    out = _both(d, p)
    assert np.array_equal(out["fused"], out["stored"])
    assert np.abs(out["fused"] - ref).max() <= MIXED_ABS


# (data vertices, data edges, edge feature dim, pattern vertices, pattern edges)
SHAPES = [(300, 3000, 17, 6, 10), (1000, 127, 17, 4, 5), (2000, 20000, 1, 5, 8),
          (2000, 20001, 3, 8, 16), (5000, 60000, 24, 10, 33), (3000, 40000, 17, 16, 64),
          (4000, 50000, 13, 12, 48), (2500, 30000, 8, 3, 1)]


@pytest.mark.parametrize("dn,de,ke,pn,pe", SHAPES)
def test_fused_shapes(cuda, dn, de, ke, pn, pe):
    d = graph.gen_er(dn, de - pe, kv=13, ke=ke, seed=dn + de)
    d, p, _, _ = graph.plant(d, pn, pe, 0.05, seed=ke)
    ref = oracle.match(d, p)
    out = _both(d, p)
    assert np.array_equal(out["fused"], out["stored"])
    assert np.abs(out["fused"] - ref).max() <= MIXED_ABS


def _hub_graph(seed=0, n_in=20000):
    """R-MAT 14 (16/32 planted) plus a vertex with n_in in-edges and as many
    out-edges: its in-edges cross many chunks of tiles."""
    d, p, _ = graph.workload("rmat14_16_32")
    rng = np.random.default_rng(seed)
    n = d.num_nodes
    hub = 7
    s = np.concatenate([np.asarray(d.srcs, np.int64), np.full(n_in, hub), rng.integers(0, n, n_in)])
    t = np.concatenate([np.asarray(d.dsts, np.int64), rng.integers(0, n, n_in), np.full(n_in, hub)])
    ef = np.concatenate([np.asarray(d.edge_feats), rng.normal(size=(2 * n_in, d.edge_feats.shape[1]))])
    return graph.Graph(np.asarray(d.node_feats), ef, s, t), p


def test_fused_hub_chunks(cuda):
    d, p = _hub_graph()
    ref = oracle.match(d, p)
    out = _both(d, p)
    assert np.array_equal(out["fused"], out["stored"])
    assert np.abs(out["fused"] - ref).max() <= MIXED_ABS


def test_fused_rmat16(cuda):
    """R-MAT 16 with a 32/64 pattern (the benchmark's pattern shape) against the
    oracle and the stored path (the default)."""
    d, p, truth = graph.workload("rmat16_32_64")
    ref = oracle.match(d, p)
    data = matcher.DataGraph(d)
    mu = matcher.Plan(data, p, "mixed", edge_kernel="fused").run().cpu().numpy()
    st = matcher.Plan(data, p, "mixed").run().cpu().numpy()
    assert np.array_equal(mu, st)
    assert np.abs(mu - ref).max() <= MIXED_ABS
    assert all(int(mu[:, i].argmax()) == int(truth[i]) for i in range(p.num_nodes))


def test_fused_unsupported_shape(cuda):
    d = graph.gen_er(200, 1000, kv=13, ke=30, seed=1)
    d, p, _, _ = graph.plant(d, 4, 6, 0.05, seed=1)
    data = matcher.DataGraph(d)
    with pytest.raises(AcgError) as e:
        matcher.Plan(data, p, "mixed", edge_kernel="fused")
    assert e.value.status == 5
    # the default reads the stored matrix
    ref = oracle.match(d, p)
    mu = matcher.Plan(data, p, "mixed").run().cpu().numpy()
    assert np.abs(mu - ref).max() <= MIXED_ABS
