"""The oracle (CPU restatement of the reference) pinned against the reference itself."""
import numpy as np
import pytest

from conftest import golden_names, load_golden
from oracle import oracle
from application_classification_gb300 import graph


@pytest.mark.parametrize("name", golden_names())
def test_oracle_matches_reference_golden(name):
    """mu of the restatement vs the exact doubles the reference printed."""
    d, p, ref = load_golden(name)
    mu = oracle.match(d, p)
    scale = max(1.0, np.abs(ref).max())
    assert np.abs(mu - ref).max() <= 1e-12 * scale
    assert (mu.argmax(1) == ref.argmax(1)).all()


@pytest.mark.skipif(not oracle.reference_available(), reason="reference CPU build not present")
@pytest.mark.parametrize("seed", [21, 22])
def test_oracle_matches_reference_fresh(seed):
    """Fresh seeded cases run through the reference binary itself."""
    d = graph.gen_er(400, 5000, seed=seed)
    d, p, _, _ = graph.plant(d, 7, 12, 0.05, seed=seed)
    ref = oracle.reference_match(d, p)
    mu = oracle.match(d, p)
    assert np.abs(mu - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())


def test_oracle_thread_count_invariant():
    d, p, _ = load_golden("er300")
    a = oracle.match(d, p, threads=1)
    b = oracle.match(d, p, threads=4)
    assert np.array_equal(a, b)


def test_oracle_num_iters():
    d, p, ref = load_golden("tiny")
    full = oracle.match(d, p, num_iters=-1)
    assert np.array_equal(full, oracle.match(d, p, num_iters=p.num_nodes))
    zero = oracle.match(d, p, num_iters=0)
    # zero iterations: MU = L(-cdist) (main.cu:112,117), columns sum to one
    assert np.allclose(np.exp(zero).sum(0), 1.0)


def test_oracle_rejects_bad_index():
    d, p, _ = load_golden("tiny")
    bad = graph.Graph(d.node_feats, d.edge_feats, d.srcs.copy(), d.dsts.copy())
    bad.dsts[0] = d.num_nodes
    with pytest.raises(ValueError):
        oracle.match(bad, p)
