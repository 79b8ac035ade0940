"""Many patterns against one data graph (acg_batch): every member's mu equals
its own single-pattern match (the groups are disjoint unions), for patterns
packed together, patterns too wide to share a group, a data graph whose quirk
coverage spans many columns, and the C-null option; the captured CUDA graph
relaunches to the same result."""
import numpy as np
import pytest

from oracle import oracle
from application_classification_gb300 import graph, matcher
from application_classification_gb300._lib import AcgError

pytestmark = pytest.mark.gpu

FP64_REL = 1e-10


def _batch_vs_single(d, pats, prec, tol_abs=None, autotune=False, cnull=False):
    dg = matcher.DataGraph(d)
    b = matcher.Batch(dg, pats, prec, autotune=autotune, cnull=cnull)
    outs = [o.cpu().numpy() for o in b.run()]
    info = b.info()
    assert info["patterns"] == len(pats) and info["groups"] < len(pats)
    for p, mu in zip(pats, outs):
        one = matcher.Plan(dg, p, prec, cnull=cnull).run().cpu().numpy()
        tol = FP64_REL * max(1.0, np.abs(one).max()) if tol_abs is None else tol_abs
        assert np.abs(mu - one).max() <= tol
    return dg, b, outs


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_batch_members_equal_single_matches(cuda, prec):
    d, pats, _ = graph.batch_workload(11, 10, seed=5)
    _batch_vs_single(d, pats, prec, None if prec == "fp64" else 2e-5)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_batch_cnull_members_equal_single_matches(cuda, prec):
    """The C-null term in a batch: each member's normaliser runs over its own
    pattern edges, so it equals the member's single match with the option."""
    d, pats, _ = graph.batch_workload(11, 10, seed=5)
    _batch_vs_single(d, pats, prec, None if prec == "fp64" else 2e-5, cnull=True)


def test_batch_cnull_fp64_vs_oracle(cuda):
    d, pats, _ = graph.batch_workload(10, 6, seed=7)
    dg = matcher.DataGraph(d)
    outs = [o.cpu().numpy() for o in matcher.Batch(dg, pats, "fp64", cnull=True).run()]
    for p, mu in zip(pats, outs):
        ref = oracle.match(d, p, cnull=True)
        assert np.abs(mu - ref).max() <= FP64_REL * max(1.0, np.abs(ref).max())


def test_batch_fp64_vs_oracle(cuda):
    d, pats, _ = graph.batch_workload(10, 6, seed=7)
    dg = matcher.DataGraph(d)
    outs = [o.cpu().numpy() for o in matcher.Batch(dg, pats, "fp64").run()]
    for p, mu in zip(pats, outs):
        ref = oracle.match(d, p)
        assert np.abs(mu - ref).max() <= FP64_REL * max(1.0, np.abs(ref).max())


def test_batch_quirk_spans_columns(cuda):
    # few edges per vertex: Pn * Dn covers many columns of every pattern
    d = graph.gen_er(400, 900, seed=11)
    pats = []
    for i, (pn, pe) in enumerate([(6, 10), (9, 14), (5, 7), (12, 20)]):
        d, p, _, _ = graph.plant(d, pn, pe, 0.05, seed=40 + i)
        pats.append(p)
    dg = matcher.DataGraph(d)
    outs = [o.cpu().numpy() for o in matcher.Batch(dg, pats, "fp64").run()]
    for p, mu in zip(pats, outs):
        ref = oracle.match(d, p)
        assert np.abs(mu - ref).max() <= FP64_REL * max(1.0, np.abs(ref).max())


def test_batch_relaunch_and_num_iters(cuda):
    d, pats, _ = graph.batch_workload(10, 5, seed=9)
    dg = matcher.DataGraph(d)
    b = matcher.Batch(dg, pats, "mixed", num_iters=3)
    first = [o.cpu().numpy().copy() for o in b.run()]
    again = [o.cpu().numpy() for o in b.run()]  # the captured graph, launched again
    for x, y in zip(first, again):
        assert np.array_equal(x, y)
    for p, mu in zip(pats, first):
        one = matcher.Plan(dg, p, "mixed", num_iters=3).run().cpu().numpy()
        assert np.abs(mu - one).max() <= 2e-5


def test_batch_rejects_bad_pattern(cuda):
    d, pats, _ = graph.batch_workload(9, 2, seed=2)
    bad = graph.gen_er(5, 6, kv=4, ke=17, seed=1)  # vertex features of another width
    with pytest.raises(AcgError):
        matcher.Batch(matcher.DataGraph(d), [pats[0], bad], "fp64")


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_batch_autotune(cuda, prec):
    """The autotuned grouping (measured cost model, dynamic programming over
    the patterns sorted by iteration count, a measured launch shape) keeps
    every member equal to its single match, and reports its model."""
    d, pats, _ = graph.batch_workload(12, 16, seed=9)
    # mixed: the tuned launch shape changes the order of the FP32 partial sums;
    # member and single match are each within ~2e-5 of FP64
    _, b, outs = _batch_vs_single(d, pats, prec, None if prec == "fp64" else 5e-5, autotune=True)
    info = b.info()
    assert info["autotuned"] == 1
    assert info["iter_ms_per_column"] >= 0 and info["once_ms_fixed"] >= 0
    assert info["predicted_ms"] > 0
    assert info["edge_blocks_per_sm"] in (0, 2) and info["vertex_blocks_per_sm"] in (0, 1)
    assert 1 <= info["groups"] <= len(pats)
    assert info["ms_last"] > 0
