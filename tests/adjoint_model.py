"""numpy model of the adjoint the CUDA backward implements (test infrastructure).

Forward: the restructured iteration of the kernels (see the header of
application_classification_gb300/csrc/acg_bp.cu), unshifted, FP64, recording
every state.  Backward: reverse mode through the same steps, with the
conventions of the kernels:
  * max(fill, b): the gradient goes to b when b > fill, else to the fill;
  * a column maximum (the fills' max_v) routes to its smallest maximal index;
  * a segmented maximum over a vertex's edges routes to its first maximal edge
    in CSR order (increasing original edge id);
  * log-sum-exps route through their softmax weights.
forward() and backward() are compared with torch autograd (adjoint_ref.py) by
tests/test_adjoint_model.py, on the CPU.
"""
import numpy as np

from kernel_algebra import lse


def _cdist(a, b):
    return np.sqrt(((a[:, None, :] - b[None, :, :]) ** 2).sum(-1))


def _softmax_cols(x):
    m = np.max(np.where(np.isfinite(x), x, -np.inf), axis=0, keepdims=True)
    m = np.where(np.isfinite(m), m, 0.0)
    w = np.exp(x - m)
    s = w.sum(0, keepdims=True)
    return np.where(s > 0, w / np.where(s > 0, s, 1), 0.0)


def _seg_argmax(vals, keys, n):
    """([n][Q] maxima, [n][Q] index of the first row e (in increasing e) with
    keys[e] == v and the largest vals[e, q]; -1 where v has no rows)."""
    De, Q = vals.shape
    best = np.full((n, Q), -np.inf)
    arg = np.full((n, Q), -1, dtype=np.int64)
    for e in range(De):
        v = keys[e]
        upd = vals[e] > best[v]
        best[v] = np.where(upd, vals[e], best[v])
        arg[v] = np.where(upd, e, arg[v])
    return best, arg


def forward(d, p, iters=None):
    """Recorded forward; returns (mu, rec)."""
    x, xe = np.asarray(d.node_feats, float), np.asarray(d.edge_feats, float)
    y, ye = np.asarray(p.node_feats, float), np.asarray(p.edge_feats, float)
    s, t = np.asarray(d.srcs).astype(np.int64), np.asarray(d.dsts).astype(np.int64)
    ps, pd = np.asarray(p.srcs).astype(np.int64), np.asarray(p.dsts).astype(np.int64)
    Dn, De, Pn, Pe = len(x), len(xe), len(y), len(ye)
    T = Pn if iters is None else iters
    dV, dE = _cdist(x, y), _cdist(xe, ye)
    CV = dV - lse(dV, 0)
    MU0 = -dV - lse(-dV, 0)
    lim = Pn * Dn
    cov = (np.arange(Pe)[None, :] * De + np.arange(De)[:, None]) < lim
    buf = np.where(cov, -dE, 0.0)
    lbuf = lse(buf, 0)
    Rb, Rarg = _seg_argmax(buf, s, Dn)
    Fb, Farg = _seg_argmax(buf, t, Dn)
    outdeg = np.bincount(s, minlength=Dn) > 0
    indeg = np.bincount(t, minlength=Dn) > 0
    negmin, dEargmin = _seg_argmax(-dE, s, Dn)
    dEmin = -negmin
    with np.errstate(divide="ignore"):
        B = np.full((Dn, Pe), -np.inf)
        for q in range(Pe):
            m = np.full(Dn, -np.inf)
            np.maximum.at(m, s, -dE[:, q])
            acc = np.zeros(Dn)
            np.add.at(acc, s, np.exp(-dE[:, q] - m[s]))
            B[:, q] = np.where(outdeg, np.log(np.where(acc > 0, acc, 1)) + m, -np.inf)
    vfmax0 = MU0[:, pd].max(0)
    vrmax0 = MU0[:, ps].max(0)
    R0b = np.where(outdeg[:, None], Rb - lbuf, -np.inf)
    F0b = np.where(indeg[:, None], Fb - lbuf, -np.inf)
    R0 = np.maximum(vfmax0, R0b)
    F0 = np.maximum(vrmax0, F0b)
    rec = dict(x=x, xe=xe, y=y, ye=ye, s=s, t=t, ps=ps, pd=pd, dV=dV, dE=dE, CV=CV, MU0=MU0,
               cov=cov, buf=buf, lbuf=lbuf, Rarg=Rarg, Farg=Farg, outdeg=outdeg, indeg=indeg,
               dEmin=dEmin, dEargmin=dEargmin, B=B, vfmax0=vfmax0, vrmax0=vrmax0, R0b=R0b, F0b=F0b,
               T=T, Dn=Dn, De=De, Pn=Pn, Pe=Pe)
    MU = [MU0]
    S = [np.zeros(Pn)]
    F, R = [F0], [R0]
    VF = [MU0[:, pd] - F0]
    VR = [MU0[:, ps] - R0]
    st = []
    for it in range(1, T + 1):
        vf, vr = VF[-1], VR[-1]
        mVF, mVR = vf.max(0), vr.max(0)
        lR, lF = lse(vf + B, 0), lse(vr + B, 0)
        aR = mVF - S[-1][pd]
        aF = mVR - S[-1][ps]
        with np.errstate(invalid="ignore"):
            bR = vf - dEmin - lR
        bR = np.where(outdeg[:, None], bR, -np.inf)
        Mv, Marg = _seg_argmax(vr[s] - dE, t, Dn)
        bF = Mv - lF
        Rn, Fn = np.maximum(aR, bR), np.maximum(aF, bF)
        MUn = -CV.copy()
        np.add.at(MUn.T, pd, Fn.T)
        np.add.at(MUn.T, ps, Rn.T)
        Sn = lse(MUn, 0)
        st.append(dict(mVF=mVF, mVR=mVR, lR=lR, lF=lF, aR=aR, aF=aF, bR=bR, bF=bF, Marg=Marg,
                       vfarg=np.argmax(vf, 0), vrarg=np.argmax(vr, 0)))
        F.append(Fn), R.append(Rn), MU.append(MUn), S.append(Sn)
        VF.append(MUn[:, pd] - Fn)
        VR.append(MUn[:, ps] - Rn)
    rec.update(MU=MU, S=S, F=F, R=R, VF=VF, VR=VR, st=st)
    return MU[-1] - S[-1], rec


def backward(rec, gmu):
    """Gradients of sum(gmu * mu) w.r.t. (data node, data edge, pattern node,
    pattern edge) features."""
    T, Dn, De, Pn, Pe = rec["T"], rec["Dn"], rec["De"], rec["Pn"], rec["Pe"]
    s, t, ps, pd = rec["s"], rec["t"], rec["ps"], rec["pd"]
    MU, S, VF, VR, B = rec["MU"], rec["S"], rec["VF"], rec["VR"], rec["B"]
    gMU = gmu - _softmax_cols(MU[T]) * gmu.sum(0)
    gFd = np.zeros((Dn, Pe))
    gRd = np.zeros((Dn, Pe))
    gCV = np.zeros((Dn, Pn))
    gdEmin = np.zeros((Dn, Pe))
    gB = np.zeros((Dn, Pe))
    gdE = np.zeros((De, Pe))
    if T == 0:
        # mu is the prior MU0 itself (normalised: S(0) is identically zero)
        gMU0 = gmu.copy()
        gF0 = np.zeros((Dn, Pe))
        gR0 = np.zeros((Dn, Pe))
    for it in range(T, 0, -1):
        k = rec["st"][it - 1]
        gF = gMU[:, pd] + gFd
        gR = gMU[:, ps] + gRd
        gCV -= gMU
        sR = k["bR"] > k["aR"]
        sF = k["bF"] > k["aF"]
        gbR = np.where(sR, gR, 0.0)
        gbF = np.where(sF, gF, 0.0)
        gaR = np.where(sR, 0.0, gR).sum(0)
        gaF = np.where(sF, 0.0, gF).sum(0)
        glR, glF = -gbR.sum(0), -gbF.sum(0)
        gdEmin -= gbR
        gVF = gbR.copy()
        gVR = np.zeros((Dn, Pe))
        for q in range(Pe):  # the segmented maximum: route to the argmax edge
            for v in range(Dn):
                e = k["Marg"][v, q]
                if e >= 0 and gbF[v, q] != 0.0:
                    gVR[s[e], q] += gbF[v, q]
                    gdE[e, q] -= gbF[v, q]
        gVF[k["vfarg"], np.arange(Pe)] += gaR
        gVR[k["vrarg"], np.arange(Pe)] += gaF
        gS = np.zeros(Pn)
        np.add.at(gS, pd, -gaR)
        np.add.at(gS, ps, -gaF)
        w = _softmax_cols(VF[it - 1] + B)
        w2 = _softmax_cols(VR[it - 1] + B)
        gVF += glR * w
        gVR += glF * w2
        gB += glR * w + glF * w2
        gM = np.zeros((Dn, Pn))
        np.add.at(gM.T, pd, gVF.T)
        np.add.at(gM.T, ps, gVR.T)
        if it - 1 >= 1:
            gM += gS * _softmax_cols(MU[it - 1])
            gMU = gM
            gFd, gRd = -gVF, -gVR
        else:
            gMU0 = gM
            gF0, gR0 = -gVF, -gVR
    # init messages: R0 = max(vfmax0, Rbuf - lbuf), F0 = max(vrmax0, Fbuf - lbuf)
    sR0 = rec["R0b"] > rec["vfmax0"]
    sF0 = rec["F0b"] > rec["vrmax0"]
    gRb = np.where(sR0, gR0, 0.0)
    gFb = np.where(sF0, gF0, 0.0)
    glbuf = -gRb.sum(0) - gFb.sum(0)
    gvf0 = np.where(sR0, 0.0, gR0).sum(0)
    gvr0 = np.where(sF0, 0.0, gF0).sum(0)
    MU0 = rec["MU0"]
    for q in range(Pe):
        gMU0[np.argmax(MU0[:, pd[q]]), pd[q]] += gvf0[q]
        gMU0[np.argmax(MU0[:, ps[q]]), ps[q]] += gvr0[q]
    cov = rec["cov"]
    for arg, gb in ((rec["Rarg"], gRb), (rec["Farg"], gFb)):
        for q in range(Pe):
            for v in range(Dn):
                e = arg[v, q]
                if e >= 0 and gb[v, q] != 0.0 and cov[e, q]:
                    gdE[e, q] -= gb[v, q]  # buf = -dE where covered
    wb = _softmax_cols(rec["buf"])
    gdE -= np.where(cov, glbuf * wb, 0.0)
    # static: dEmin (argmin routing), B (softmax over out-edges)
    for q in range(Pe):
        for v in range(Dn):
            e = rec["dEargmin"][v, q]
            if e >= 0:
                gdE[e, q] += gdEmin[v, q]
    dE = rec["dE"]
    with np.errstate(invalid="ignore"):
        wB = np.exp(-dE - B[s])
    gdE -= np.where(np.isfinite(B[s]), gB[s] * wB, 0.0)
    # MU0 = -dV - lse(-dV), CV = dV - lse(dV)
    dV = rec["dV"]
    gdV = -gMU0 + _softmax_cols(-dV) * gMU0.sum(0)
    gdV += gCV - _softmax_cols(dV) * gCV.sum(0)

    def cd_back(g, a, b, dist):  # d = ||a - b||
        with np.errstate(invalid="ignore", divide="ignore"):
            r = np.where(dist > 0, g / dist, 0.0)
        diff = a[:, None, :] - b[None, :, :]
        return (r[:, :, None] * diff).sum(1), -(r[:, :, None] * diff).sum(0)

    gx, gy = cd_back(gdV, rec["x"], rec["y"], dV)
    gxe, gye = cd_back(gdE, rec["xe"], rec["ye"], dE)
    return gx, gxe, gy, gye
