"""FP64 PyTorch re-implementation of the reference matcher, differentiable in
the four feature arrays (test infrastructure for the adjoint).

It follows the reference's own passes (src/main.cu:104-247, src/ac.hxx:17-186)
rather than the kernels' restructured algebra, so that it checks both: the
quirk buffer of main.cu:113-114 (only the first Pn*Dn flat elements of the
[Pe][De] RE/FE buffers hold -CE, the rest are zero), the row log-softmaxes
L(x) = x - log(sum(exp(x))) over the data axis (ac.hxx:77-113), the edge
max-reductions (ac.hxx:115-149) and ComputeMU (ac.hxx:151-186).  Maxima route
their gradient to one maximal element (torch's amax/scatter_reduce choose);
ties have measure zero for continuous features.
"""
import torch


def _cdist(a, b):
    # [na][nb] = ||a_i - b_j||_2, the difference form of ac.hxx:33-56
    return torch.sqrt(((a[:, None, :] - b[None, :, :]) ** 2).sum(-1))


def _L(x):
    return x - torch.logsumexp(x, dim=-1, keepdim=True)


def _edge_max(base, vals, nodes, n):
    # out[r][v] = max(base[r], max_{e: nodes[e] = v} vals[r][e])  (ac.hxx:115-149)
    out = base[:, None].expand(-1, n).clone()
    idx = nodes[None, :].expand(vals.shape[0], -1)
    return out.scatter_reduce(1, idx, vals, reduce="amax", include_self=True)


def match(dnf, def_, pnf, pef, srcs, dsts, psrc, pdst, iters=None, cnull=False):
    """mu [Dn][Pn] (float64 tensor) from the four feature tensors; srcs/dsts and
    psrc/pdst are int64 tensors of the data and pattern endpoints.  cnull: the
    optional C-null term as test.py:93-97 and 139-140 state it (the reference
    leaves it out): cn_q = max(||pe_q||, max_e L(ce)[q][e]) normalised by a
    log-softmax over q, subtracted from both fills in every iteration."""
    Dn, Pn, Pe, De = dnf.shape[0], pnf.shape[0], pef.shape[0], def_.shape[0]
    T = Pn if iters is None else iters
    cv_t = _cdist(pnf, dnf)                     # [Pn][Dn]
    ce_t = _cdist(pef, def_)                    # [Pe][De]
    mu_t = -cv_t
    nneg = min(Pn * Dn, Pe * De)
    flat = torch.arange(Pe * De).reshape(Pe, De)
    buf = torch.where(flat < nneg, -ce_t, torch.zeros_like(ce_t))
    cv_t = _L(cv_t)
    mu_t = _L(mu_t)
    ce_t = _L(ce_t)
    re_t = _L(buf)
    fe_t = _L(buf)
    vr_t = mu_t[psrc]
    vf_t = mu_t[pdst]
    vfmax = vf_t.amax(1)
    vrmax = vr_t.amax(1)
    rmax_t = _edge_max(vfmax, re_t, srcs, Dn)
    fmax_t = _edge_max(vrmax, fe_t, dsts, Dn)
    cn = None
    if cnull and Pe > 0:
        cn = torch.sqrt((pef ** 2).sum(-1))
        if De > 0:
            cn = torch.maximum(cn, ce_t.amax(1))
        cn = cn - torch.logsumexp(cn, dim=0)
    for _ in range(T):
        vf_t = mu_t[pdst] - fmax_t
        vr_t = mu_t[psrc] - rmax_t
        fe_t = vr_t[:, srcs] - ce_t
        re_t = vf_t[:, srcs] - ce_t
        vfmax = vf_t.amax(1)
        if cn is not None:
            vfmax = vfmax - cn
        re_t = _L(re_t)
        rmax_t = _edge_max(vfmax, re_t, srcs, Dn)
        vrmax = vr_t.amax(1)
        if cn is not None:
            vrmax = vrmax - cn
        fe_t = _L(fe_t)
        fmax_t = _edge_max(vrmax, fe_t, dsts, Dn)
        mu_t = -cv_t
        mu_t = mu_t.index_add(0, pdst, fmax_t).index_add(0, psrc, rmax_t)
        mu_t = _L(mu_t)
    return mu_t.T.contiguous()


def match_graphs(d, p, iters=None, requires_grad=True, cnull=False):
    """match() on host graphs (graph.Graph); returns (mu, [dnf, def, pnf, pef])."""
    import numpy as np

    t = lambda a: torch.tensor(np.asarray(a), dtype=torch.float64, requires_grad=requires_grad)
    i = lambda a: torch.tensor(np.asarray(a).astype(np.int64))
    feats = [t(d.node_feats), t(d.edge_feats), t(p.node_feats), t(p.edge_feats)]
    mu = match(*feats, i(d.srcs), i(d.dsts), i(p.srcs), i(p.dsts), iters, cnull)
    return mu, feats
