"""The match as a differentiable PyTorch function.

:class:`MatchFunction` runs the forward through ``acg_match_record`` and the
backward through ``acg_backward`` (the hand-written adjoint in
``csrc/acg_adjoint.cu``): gradients of the matching scores with respect to the
data and pattern vertex and edge features.  The reference has no backward; its
forward is ``main.cu:107-247``.  Each call prepares the data graph afresh (its
CSR orderings and, in mixed precision, the FP32 copies of the features), so
features may change between calls.  PyTorch only carries the tensors; every
kernel is the native library's, and there is no fallback.
"""
from __future__ import annotations

import torch

from .matcher import DataGraph, DeviceGraph, Plan


class MatchFunction(torch.autograd.Function):
    """mu = match(data node feats, data edge feats, pattern node feats, pattern edge feats).

    Topology (``srcs``/``dsts``, ``psrc``/``pdst``: int64 or uint64 device
    tensors) and the options are non-differentiable arguments."""

    @staticmethod
    def forward(ctx, dnf, def_, pnf, pef, srcs, dsts, psrc, pdst, precision="fp64", num_iters=-1,
                checkpoint_every=4):
        feats = [t.detach().to(torch.float64).contiguous() for t in (dnf, def_, pnf, pef)]
        dg = DeviceGraph.from_tensors(feats[0], feats[1], srcs.contiguous(), dsts.contiguous())
        pg = DeviceGraph.from_tensors(feats[2], feats[3], psrc.contiguous(), pdst.contiguous())
        data = DataGraph(dg)
        plan = Plan(data, pg, precision, num_iters)
        mu = plan.record(checkpoint_every=checkpoint_every)
        ctx.plan, ctx.data = plan, data
        ctx.dtypes = [t.dtype for t in (dnf, def_, pnf, pef)]
        return mu

    @staticmethod
    def backward(ctx, gmu):
        # the plan (and its checkpoints) lives as long as the autograd graph:
        # a retained graph may be differentiated again
        grads = ctx.plan.backward(gmu)
        out = [g.to(dt) if ctx.needs_input_grad[i] else None
               for i, (g, dt) in enumerate(zip(grads, ctx.dtypes))]
        return (*out, None, None, None, None, None, None, None)


def match(dnf, def_, pnf, pef, srcs, dsts, psrc, pdst, precision: str = "fp64",
          num_iters: int = -1, checkpoint_every: int = 4):
    """Differentiable match of device tensors; returns mu [Dn][Pn] (float64)."""
    return MatchFunction.apply(dnf, def_, pnf, pef, srcs, dsts, psrc, pdst, precision, num_iters,
                               checkpoint_every)
