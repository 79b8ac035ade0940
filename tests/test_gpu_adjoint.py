"""The CUDA adjoint (acg_match_record / acg_backward) through the C ABI.

Checked against:
  * the numpy model of the same adjoint (adjoint_model.py), which the CPU
    suite proves equal to torch autograd through an FP64 re-implementation of
    the reference's own passes (adjoint_ref.py, pinned to the golden mu);
    FP64 bar: 1e-9 relative to the largest gradient entry;
  * central finite differences of sum(gmu * mu) through acg_match (FP64);
  * itself: bit-identical for every checkpoint interval and on repeated calls
    (every reduction has a fixed order);
  * the mixed path against the FP64 gradients (FP32 belief propagation).
"""
import numpy as np
import pytest
import torch

import adjoint_model
from conftest import load_golden
from application_classification_gb300 import graph, matcher
from application_classification_gb300._lib import AcgError
from application_classification_gb300.autograd import match as amatch

pytestmark = pytest.mark.gpu

FP64_REL = 1e-9
MIXED_REL = 2e-3  # relative Frobenius norm, per feature array


def _grads(d, p, gmu, prec="fp64", iters=-1, every=4, repeat=1, cnull=False):
    data = matcher.DataGraph(d)
    plan = matcher.Plan(data, p, prec, iters, cnull=cnull)
    try:
        mu = plan.record(checkpoint_every=every)
        gs = [plan.backward(torch.from_numpy(gmu)) for _ in range(repeat)]
        torch.cuda.synchronize()
        out = mu.cpu().numpy(), [[x.cpu().numpy() for x in g] for g in gs]
    finally:
        plan.close()
        data.close()
    return out[0], out[1] if repeat > 1 else out[1][0]


def _rel(a, b):
    return np.abs(a - b).max() / max(1.0, np.abs(b).max())


def _vs_model(d, p, iters=None, seed=0, every=4):
    gmu = np.random.default_rng(seed).normal(size=(d.num_nodes, p.num_nodes))
    mu_m, rec = adjoint_model.forward(d, p, iters)
    mu, g = _grads(d, p, gmu, "fp64", -1 if iters is None else iters, every)
    assert _rel(mu, mu_m) <= 1e-10
    for a, b in zip(g, adjoint_model.backward(rec, gmu)):
        assert a.shape == b.shape
        assert _rel(a, b) <= FP64_REL, _rel(a, b)


@pytest.mark.parametrize("name", ["tiny", "irregular", "er300", "rmat9", "georgiy"])
def test_fp64_vs_model_golden(cuda, name):
    d, p, _ = load_golden(name)
    _vs_model(d, p)


@pytest.mark.parametrize("iters", [0, 1, 2, 3])
def test_fp64_vs_model_few_iterations(cuda, iters):
    d, p, _ = graph.workload("rmat8_5_9")
    _vs_model(d, p, iters, seed=iters, every=2)


def _hub_graph(seed=0):
    """200 vertices; vertex 0 has 1,500 out-edges and 1,500 in-edges (split
    into chunks by the work partition), plus 2,000 random edges."""
    rng = np.random.default_rng(seed)
    n = 200
    s = np.concatenate([np.zeros(1500, np.int64), rng.integers(1, n, 1500), rng.integers(0, n, 2000)])
    t = np.concatenate([rng.integers(1, n, 1500), np.zeros(1500, np.int64), rng.integers(0, n, 2000)])
    perm = rng.permutation(len(s))
    d = graph.Graph(rng.normal(size=(n, 13)), rng.normal(size=(len(s), 17)), s[perm], t[perm])
    d, p, _, _ = graph.plant(d, 6, 12, 0.05, seed=seed)
    return d, p


def test_fp64_vs_model_hub(cuda):
    d, p = _hub_graph()
    _vs_model(d, p)


def test_fp64_vs_model_wide_pattern(cuda):
    # Pn and padded Pe above 32: the two-columns-per-lane forms
    d, p, _ = graph.workload("rmat10_40_60")
    _vs_model(d, p, iters=3, every=2)


def test_checkpoint_interval_and_repeat_bitwise(cuda):
    d, p, _ = graph.workload("rmat10_9_18")
    gmu = np.random.default_rng(5).normal(size=(d.num_nodes, p.num_nodes))
    mu0, (g0, g1) = _grads(d, p, gmu, every=4, repeat=2)
    for a, b in zip(g0, g1):
        assert np.array_equal(a, b)
    for every in (1, 2, 3, 100):
        mu, g = _grads(d, p, gmu, every=every)
        assert np.array_equal(mu, mu0)
        for a, b in zip(g, g0):
            assert np.array_equal(a, b), every


def test_fp64_finite_differences(cuda):
    d, p, _ = graph.workload("rmat9_6_10")
    rng = np.random.default_rng(11)
    gmu = rng.normal(size=(d.num_nodes, p.num_nodes))
    _, g = _grads(d, p, gmu)
    arrays = [(d, "node_feats"), (d, "edge_feats"), (p, "node_feats"), (p, "edge_feats")]

    def f():
        return float((matcher.match(d, p, "fp64") * gmu).sum())

    h = 1e-5
    for k, (gr, attr) in enumerate(arrays):
        a = getattr(gr, attr)
        scale = max(1e-3, np.abs(g[k]).max())
        # the entries with the largest gradients, and a few random ones
        flat = np.argsort(-np.abs(g[k]).ravel())[:3].tolist() + rng.integers(0, a.size, 3).tolist()
        for i in flat:
            idx = np.unravel_index(i, a.shape)
            x0 = a[idx]
            a[idx] = x0 + h
            fp = f()
            a[idx] = x0 - h
            fm = f()
            a[idx] = x0
            fd = (fp - fm) / (2 * h)
            assert abs(fd - g[k][idx]) <= 1e-5 * scale, (attr, idx, fd, g[k][idx])


@pytest.mark.parametrize("case", ["rmat10_9_18", "er300"])
def test_mixed_vs_fp64(cuda, case):
    if case == "er300":
        d, p, _ = load_golden(case)
    else:
        d, p, _ = graph.workload(case)
    gmu = np.random.default_rng(3).normal(size=(d.num_nodes, p.num_nodes))
    _, g64 = _grads(d, p, gmu, "fp64")
    _, g32 = _grads(d, p, gmu, "mixed")
    for a, b in zip(g32, g64):
        err = np.linalg.norm(a - b) / max(1e-30, np.linalg.norm(b))
        assert err <= MIXED_REL, err


def test_autograd_function(cuda):
    d, p, _ = load_golden("er300")
    dev = cuda
    t = lambda a: torch.tensor(a, dtype=torch.float64, device=dev, requires_grad=True)
    i = lambda a: torch.tensor(a.astype(np.int64), device=dev)
    feats = [t(d.node_feats), t(d.edge_feats), t(p.node_feats), t(p.edge_feats)]
    mu = amatch(*feats, i(d.srcs), i(d.dsts), i(p.srcs), i(p.dsts))
    gmu = torch.randn(mu.shape, dtype=torch.float64, device=dev, generator=torch.Generator(dev).manual_seed(0))
    (mu * gmu).sum().backward()
    mu_m, rec = adjoint_model.forward(d, p)
    assert _rel(mu.detach().cpu().numpy(), mu_m) <= 1e-10
    for f, b in zip(feats, adjoint_model.backward(rec, gmu.cpu().numpy())):
        assert _rel(f.grad.cpu().numpy(), b) <= FP64_REL


def test_autograd_gradcheck_tiny(cuda):
    d, p, _ = load_golden("tiny")
    dev = cuda
    i = lambda a: torch.tensor(a.astype(np.int64), device=dev)
    topo = (i(d.srcs), i(d.dsts), i(p.srcs), i(p.dsts))
    args = [torch.tensor(a, dtype=torch.float64, device=dev, requires_grad=True)
            for a in (d.node_feats, d.edge_feats, p.node_feats, p.edge_feats)]
    assert torch.autograd.gradcheck(lambda a, b, c, e: amatch(a, b, c, e, *topo), args,
                                    eps=1e-6, atol=1e-6, rtol=1e-5)


def test_backward_errors(cuda):
    d, p, _ = load_golden("irregular")
    data = matcher.DataGraph(d)
    plan = matcher.Plan(data, p, "fp64")
    g = torch.zeros((d.num_nodes, p.num_nodes), dtype=torch.float64)
    with pytest.raises(AcgError) as e:
        plan.backward(g)  # no record yet
    assert e.value.status == 1
    plan.record()
    plan.backward(g)
    plan.close()
    d2, p2, _ = graph.workload("rmat9_66_70")  # 66 pattern vertices: above the adjoint's limit
    data2 = matcher.DataGraph(d2)
    plan2 = matcher.Plan(data2, p2, "fp64", num_iters=1)
    with pytest.raises(AcgError) as e:
        plan2.record()
    assert e.value.status == 5
    plan2.close()
    data.close()
    data2.close()


def _planted_gmu(d, p, truth):
    g = np.zeros((d.num_nodes, p.num_nodes))
    g[np.asarray(truth, dtype=np.int64), np.arange(p.num_nodes)] = 1.0
    return g


def test_rmat12_planted_loss_vs_autograd_reference(cuda):
    """Loss = sum of mu (the log assignment probability) over the planted
    pairs, RMAT scale 12 with a 12/24 pattern: the FP64 and mixed gradients
    against torch autograd through the reference's own passes (FP64, CPU)."""
    import adjoint_ref

    d, p, truth = graph.workload("rmat12")
    gmu = _planted_gmu(d, p, truth)
    mu_t, feats = adjoint_ref.match_graphs(d, p)
    (mu_t * torch.from_numpy(gmu)).sum().backward()
    ref = [f.grad.numpy() for f in feats]
    mu64, g64 = _grads(d, p, gmu, "fp64")
    assert _rel(mu64, mu_t.detach().numpy()) <= 1e-10
    for a, b in zip(g64, ref):
        assert _rel(a, b) <= FP64_REL, _rel(a, b)
    _, g32 = _grads(d, p, gmu, "mixed")
    for a, b in zip(g32, ref):
        assert np.linalg.norm(a - b) / np.linalg.norm(b) <= MIXED_REL


def test_rmat12_finite_differences_200(cuda):
    """FP64 central differences on 200 random coordinates (50 per feature
    array), perturbing the device features in place under one plan."""
    d, p, truth = graph.workload("rmat12")
    gmu = torch.from_numpy(_planted_gmu(d, p, truth)).to(cuda)
    data = matcher.DataGraph(d)
    plan = matcher.Plan(data, p, "fp64")
    try:
        plan.record()
        g = [x.cpu().numpy() for x in plan.backward(gmu)]
        arrays = [data.dev.node_feats, data.dev.edge_feats, plan.pat.node_feats, plan.pat.edge_feats]
        rng = np.random.default_rng(12)
        mu = torch.empty((d.num_nodes, p.num_nodes), dtype=torch.float64, device=cuda)

        def f():
            plan.run(mu)
            return float((mu * gmu).sum())

        h = 1e-5
        for k, a in enumerate(arrays):
            scale = max(1e-3, np.abs(g[k]).max())
            flat = a.view(-1)
            for i in rng.integers(0, flat.numel(), 50).tolist():
                x0 = flat[i].item()
                flat[i] = x0 + h
                fp = f()
                flat[i] = x0 - h
                fm = f()
                flat[i] = x0
                fd = (fp - fm) / (2 * h)
                idx = np.unravel_index(i, tuple(a.shape))
                assert abs(fd - g[k][idx]) <= 1e-5 * scale, (k, idx, fd, g[k][idx])
    finally:
        plan.close()
        data.close()


@pytest.mark.parametrize("name", ["irregular", "er300"])
def test_cnull_vs_autograd_reference(cuda, name):
    """The C-null option: the term is made of the pattern edge features' norms
    (its log-softmax alternative never exceeds them), so its gradient reaches
    those features.  FP64 against torch autograd through the reference's
    passes with the term, mixed within its bound, and central differences on
    the pattern edge features."""
    import adjoint_ref

    d, p, _ = load_golden(name)
    gmu = np.random.default_rng(4).normal(size=(d.num_nodes, p.num_nodes))
    mu_t, feats = adjoint_ref.match_graphs(d, p, cnull=True)
    (mu_t * torch.from_numpy(gmu)).sum().backward()
    ref = [f.grad.numpy() for f in feats]
    mu64, g64 = _grads(d, p, gmu, "fp64", cnull=True)
    assert _rel(mu64, mu_t.detach().numpy()) <= 1e-10
    for a, b in zip(g64, ref):
        assert _rel(a, b) <= FP64_REL, _rel(a, b)
    _, g32 = _grads(d, p, gmu, "mixed", cnull=True)
    # relative to each array's gradient, or to a thousandth of the largest one
    # where an array's gradient all but vanishes (the fills win everywhere)
    big = max(np.linalg.norm(b) for b in ref)
    for a, b in zip(g32, ref):
        assert np.linalg.norm(a - b) <= MIXED_REL * max(np.linalg.norm(b), 1e-3 * big)

    def f():
        return float((matcher.match(d, p, "fp64", cnull=True) * gmu).sum())

    h = 1e-5
    a = p.edge_feats
    scale = max(1e-3, np.abs(g64[3]).max())
    for i in np.argsort(-np.abs(g64[3]).ravel())[:4].tolist():
        idx = np.unravel_index(i, a.shape)
        x0 = a[idx]
        a[idx] = x0 + h
        fp = f()
        a[idx] = x0 - h
        fm = f()
        a[idx] = x0
        assert abs((fp - fm) / (2 * h) - g64[3][idx]) <= 1e-5 * scale
