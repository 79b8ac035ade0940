"""numpy model of the algebra the GPU kernels use (test infrastructure).

The kernels do not run the reference's passes literally: they use exact
identities that remove every per-edge exp/log from the BP loop (see the header
of application_classification_gb300/csrc/acg_bp.cu).  This model states those
identities in numpy so that tests can check, on the CPU, that they reproduce
the reference (golden fixtures) -- independently of any CUDA code.
"""
import numpy as np
from scipy.spatial.distance import cdist


def lse(x, axis=0):
    m = x.max(axis=axis, keepdims=True)
    m = np.where(np.isfinite(m), m, 0.0)
    with np.errstate(divide="ignore"):
        return (np.log(np.exp(x - m).sum(axis=axis, keepdims=True)) + m).squeeze(axis)


def seg(vals, keys, n, op, init):
    out = np.full((n,) + vals.shape[1:], init, dtype=vals.dtype)
    op.at(out, keys, vals)
    return out


def match(d, p, num_iters=-1, dt=np.float64, cnull=False):
    Dn, De, Pn, Pe = d.num_nodes, d.num_edges, p.num_nodes, p.num_edges
    iters = Pn if num_iters < 0 else num_iters
    s, t = d.srcs.astype(np.int64), d.dsts.astype(np.int64)
    ps, pd = p.srcs.astype(np.int64), p.dsts.astype(np.int64)
    dV = cdist(d.node_feats, p.node_feats)                 # [Dn, Pn]
    dE = cdist(d.edge_feats, p.edge_feats) if De else np.zeros((0, Pe))
    CV = dV - lse(dV, 0)                                   # L(dV)
    MU = -dV - lse(-dV, 0)                                 # L(-dV)
    # quirk buffer of main.cu:113-114 (zero past Pn*Dn flat elements)
    flat = np.arange(Pe)[None, :] * De + np.arange(De)[:, None]
    buf = np.where(flat < Pn * Dn, -dE, 0.0)
    L0 = buf - lse(buf, 0) if De else buf
    VFmax0 = MU[:, pd].max(0) if Pe else np.zeros(0)
    VRmax0 = MU[:, ps].max(0) if Pe else np.zeros(0)
    RMax = np.maximum(VFmax0, seg(L0, s, Dn, np.maximum, -np.inf))
    FMax = np.maximum(VRmax0, seg(L0, t, Dn, np.maximum, -np.inf))
    outdeg = np.bincount(s, minlength=Dn)[:, None]
    indeg = np.bincount(t, minlength=Dn)[:, None]
    mneg = seg(-dE, s, Dn, np.maximum, -np.inf)            # -dEmin
    ssum = seg(np.exp(-dE - np.where(np.isfinite(mneg[s]), mneg[s], 0)), s, Dn, np.add, 0.0)
    with np.errstate(divide="ignore"):
        B = np.log(ssum) + mneg                            # log sum_out exp(-dE)
    cn = np.zeros(Pe)
    if cnull and Pe:  # test.py:93-97: normprob(max(||pe_q||, max_e L(dE)[q]))
        cn = np.sqrt((np.asarray(p.edge_feats, float) ** 2).sum(1))
        if De:
            cn = np.maximum(cn, (dE - lse(dE, 0)).max(0))
        cn = cn - lse(cn, 0)
    MU, RMax, FMax, CVc, Bc, dEc, dEmin = (a.astype(dt) for a in (MU, RMax, FMax, CV, B, dE, -mneg))
    for _ in range(iters):
        VF = MU[:, pd] - FMax
        VR = MU[:, ps] - RMax
        VFm, VRm = VF.max(0) - cn, VR.max(0) - cn
        SR = lse((VF + Bc).astype(np.float64), 0)
        SF = lse((VR + Bc).astype(np.float64), 0)
        with np.errstate(invalid="ignore"):
            RMax = np.where(outdeg > 0, np.maximum(VFm, VF - dEmin - SR), VFm).astype(dt)
        M = seg(VR[s] - dEc, t, Dn, np.maximum, -np.inf)
        with np.errstate(invalid="ignore"):
            FMax = np.where(indeg > 0, np.maximum(VRm, M - SF), VRm).astype(dt)
        MUu = -CVc.copy()
        for q in range(Pe):
            MUu[:, pd[q]] += FMax[:, q]
            MUu[:, ps[q]] += RMax[:, q]
        MU = (MUu - lse(MUu.astype(np.float64), 0)).astype(dt)
    return MU.astype(np.float64)
