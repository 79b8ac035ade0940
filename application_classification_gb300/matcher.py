"""Python host API over the C ABI: the reference's driver flow with device-resident graphs.

The reference's ``main`` (src/main.cu:66-257) loads two graphs to the device,
runs the matcher and copies ``MU`` back.  Here:

* :class:`DeviceGraph` holds a graph's arrays on a CUDA device (what
  ``loadGraph`` does, main.cu:54-62),
* :class:`DataGraph` is ``acg_data`` (the data graph with its two CSR
  orderings, built once and shared by every pattern),
* :class:`Plan` is ``acg_plan`` (one pattern against one data graph),
* :func:`match` is the one-shot host-to-host call.

PyTorch provides device memory and streams only; every kernel is the native
library's.  There is no CPU fallback: without CUDA these raise.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .graph import Graph

PRECISIONS = {"fp64": _lib.PREC_FP64, "mixed": _lib.PREC_MIXED}
# acg_options.cdist_kernel: the mixed path's edge and vertex cost matrices
CDIST_KERNELS = {"auto": 0, "simt": 1, "tensor": 2}
# acg_options.edge_kernel: the mixed path's edge phase (costs recomputed on the
# tensor cores, or read from the stored edge cost matrix)
EDGE_KERNELS = {"auto": 0, "stored": 1, "fused": 2}


def _torch():
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("CUDA is not available: the matcher runs on the GPU only")
    return torch


def _stream_ptr(stream) -> int:
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)


class DeviceGraph:
    """A graph's four arrays on a CUDA device (f64 features, u64 endpoints)."""

    def __init__(self, g: Graph, device="cuda", pinned: bool = False, stream=None):
        torch = _torch()
        self.num_nodes, self.node_feat_dim = g.node_feats.shape
        self.num_edges, self.edge_feat_dim = g.edge_feats.shape

        def up(a, dtype):
            t = torch.from_numpy(a.view(np.int64) if a.dtype == np.uint64 else a)
            if pinned:
                t = t.pin_memory()
            return t.to(device, non_blocking=pinned)

        self.node_feats = up(g.node_feats, None)
        self.edge_feats = up(g.edge_feats, None)
        self.srcs = up(g.srcs, None)
        self.dsts = up(g.dsts, None)

    @classmethod
    def from_tensors(cls, node_feats, edge_feats, srcs, dsts) -> "DeviceGraph":
        """Wrap device tensors (f64 [N][Kv], f64 [M][Ke], int64/uint64 [M] x2)."""
        self = cls.__new__(cls)
        self.num_nodes, self.node_feat_dim = node_feats.shape
        self.num_edges, self.edge_feat_dim = edge_feats.shape
        self.node_feats, self.edge_feats, self.srcs, self.dsts = node_feats, edge_feats, srcs, dsts
        return self

    def c_graph(self) -> _lib.Graph:
        g = _lib.Graph()
        g.num_nodes, g.node_feat_dim = self.num_nodes, self.node_feat_dim
        g.num_edges, g.edge_feat_dim = self.num_edges, self.edge_feat_dim
        g.node_feats = self.node_feats.data_ptr()
        g.edge_feats = self.edge_feats.data_ptr()
        g.srcs = self.srcs.data_ptr()
        g.dsts = self.dsts.data_ptr()
        return g


class DataGraph:
    """``acg_data``: a data graph prepared for matching (CSR orderings)."""

    def __init__(self, graph, stream=None):
        self.dev = graph if isinstance(graph, DeviceGraph) else DeviceGraph(graph)
        self._c = self.dev.c_graph()
        self.handle = C.c_void_p()
        _lib.check(_lib.lib().acg_data_create(C.byref(self._c), _stream_ptr(stream),
                                              C.byref(self.handle)), "acg_data_create")

    @property
    def num_nodes(self) -> int:
        return self.dev.num_nodes

    def close(self):
        if self.handle:
            _lib.lib().acg_data_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Plan:
    """``acg_plan``: one pattern matched against one :class:`DataGraph`."""

    def __init__(self, data: DataGraph, pattern, precision: str = "fp64", num_iters: int = -1,
                 stream=None, kernel_timing: bool = False, edge_blocks_per_sm: int = 0,
                 vertex_blocks_per_sm: int = 0, cnull: bool = False, cdist_kernel: str = "auto",
                 edge_kernel: str = "auto"):
        self.data = data
        self.pat = pattern if isinstance(pattern, DeviceGraph) else DeviceGraph(pattern)
        self._c = self.pat.c_graph()
        opt = _lib.Options()
        _lib.lib().acg_options_default(C.byref(opt))
        if precision not in PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(PRECISIONS)}")
        opt.precision = PRECISIONS[precision]
        opt.num_iters = num_iters
        opt.kernel_timing = 1 if kernel_timing else 0
        opt.edge_blocks_per_sm = int(edge_blocks_per_sm)
        opt.vertex_blocks_per_sm = int(vertex_blocks_per_sm)
        opt.cnull = 1 if cnull else 0
        opt.cdist_kernel = CDIST_KERNELS[cdist_kernel]
        opt.edge_kernel = EDGE_KERNELS[edge_kernel]
        self.precision = precision
        self.handle = C.c_void_p()
        _lib.check(_lib.lib().acg_plan_create(data.handle, C.byref(self._c), C.byref(opt),
                                              _stream_ptr(stream), C.byref(self.handle)),
                   "acg_plan_create")

    def run(self, out=None, stream=None):
        """Run the match; returns (or fills) a [Dn][Pn] float64 device tensor."""
        torch = _torch()
        if out is None:
            out = torch.empty((self.data.num_nodes, self.pat.num_nodes), dtype=torch.float64,
                              device=self.data.dev.node_feats.device)
        _lib.check(_lib.lib().acg_match(self.handle, C.c_void_p(out.data_ptr()),
                                        _stream_ptr(stream)), "acg_match")
        return out

    def record(self, out=None, checkpoint_every: int = 4, stream=None):
        """:meth:`run` that also keeps the states the adjoint needs (every
        ``checkpoint_every``-th BP iteration and the last); returns mu."""
        torch = _torch()
        if out is None:
            out = torch.empty((self.data.num_nodes, self.pat.num_nodes), dtype=torch.float64,
                              device=self.data.dev.node_feats.device)
        _lib.check(_lib.lib().acg_match_record(self.handle, C.c_void_p(out.data_ptr()),
                                               int(checkpoint_every), _stream_ptr(stream)),
                   "acg_match_record")
        return out

    def backward(self, grad_mu, stream=None):
        """Gradients of sum(grad_mu * mu) for the last :meth:`record`: a tuple
        (data node, data edge, pattern node, pattern edge) of float64 tensors
        shaped like the four feature arrays."""
        torch = _torch()
        dev = self.data.dev.node_feats.device
        g = grad_mu.to(device=dev, dtype=torch.float64).contiguous()
        outs = [torch.empty(tuple(t.shape), dtype=torch.float64, device=dev)
                for t in (self.data.dev.node_feats, self.data.dev.edge_feats,
                          self.pat.node_feats, self.pat.edge_feats)]
        _lib.check(_lib.lib().acg_backward(self.handle, C.c_void_p(g.data_ptr()),
                                           *[C.c_void_p(o.data_ptr()) for o in outs],
                                           _stream_ptr(stream)), "acg_backward")
        return tuple(outs)

    def stats(self) -> dict:
        st = _lib.Stats()
        _lib.check(_lib.lib().acg_plan_stats(self.handle, C.byref(st)), "acg_plan_stats")
        return {k: getattr(st, k) for k, _ in _lib.Stats._fields_}

    def close(self):
        if self.handle:
            _lib.lib().acg_plan_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def match(data: Graph, pattern: Graph, precision: str = "fp64", num_iters: int = -1,
          device: str = "cuda", cnull: bool = False) -> np.ndarray:
    """One-shot match of host graphs; returns mu as a [Dn][Pn] float64 numpy array.

    This is the reference's whole program between reading the two graph files
    and printing ``MU`` (main.cu:71-257), through ``acg_match_graphs``."""
    torch = _torch()
    dg, pg = DeviceGraph(data, device), DeviceGraph(pattern, device)
    out = torch.empty((dg.num_nodes, pg.num_nodes), dtype=torch.float64, device=device)
    opt = _lib.Options()
    _lib.lib().acg_options_default(C.byref(opt))
    opt.precision = PRECISIONS[precision]
    opt.num_iters = num_iters
    opt.cnull = 1 if cnull else 0
    cd, cp = dg.c_graph(), pg.c_graph()
    _lib.check(_lib.lib().acg_match_graphs(C.byref(cd), C.byref(cp), C.byref(opt),
                                           C.c_void_p(out.data_ptr()), _stream_ptr(None)),
               "acg_match_graphs")
    return out.cpu().numpy()


def match_host(data: Graph, pattern: Graph, precision: str = "fp64", num_iters: int = -1,
               cnull: bool = False, out: np.ndarray | None = None) -> np.ndarray:
    """One-shot match from host memory through ``acg_match_graphs_host``: the
    arrays of ``data`` and ``pattern`` (numpy, or pinned torch tensors wrapped
    in a :class:`Graph`-like object) are copied by the library, mu comes back in
    ``out`` (a [Dn][Pn] float64 host array, allocated if None)."""
    _torch()
    opt = _lib.Options()
    _lib.lib().acg_options_default(C.byref(opt))
    opt.precision = PRECISIONS[precision]
    opt.num_iters = num_iters
    opt.cnull = 1 if cnull else 0
    if out is None:
        out = np.empty((data.num_nodes, pattern.num_nodes), dtype=np.float64)
    cd, cp = data.c_graph(), pattern.c_graph()
    _lib.check(_lib.lib().acg_match_graphs_host(C.byref(cd), C.byref(cp), C.byref(opt),
                                                C.c_void_p(out.ctypes.data if out.size else 0),
                                                _stream_ptr(None)), "acg_match_graphs_host")
    return out


class Batch:
    """``acg_batch``: many patterns matched against one :class:`DataGraph`.

    The patterns are packed into groups matched as disjoint unions and the whole
    batch runs as one CUDA graph launch per :meth:`run`."""

    def __init__(self, data: DataGraph, patterns, precision: str = "fp64", num_iters: int = -1,
                 stream=None, autotune: bool = False, edge_blocks_per_sm: int = 0,
                 cnull: bool = False):
        self.data = data
        self.pats = [p if isinstance(p, DeviceGraph) else DeviceGraph(p) for p in patterns]
        arr = (_lib.Graph * len(self.pats))(*[p.c_graph() for p in self.pats])
        self._arr = arr
        opt = _lib.Options()
        _lib.lib().acg_options_default(C.byref(opt))
        if precision not in PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(PRECISIONS)}")
        opt.precision = PRECISIONS[precision]
        opt.num_iters = num_iters
        opt.autotune = 1 if autotune else 0
        opt.edge_blocks_per_sm = int(edge_blocks_per_sm)  # the autotuner picks its own
        opt.cnull = 1 if cnull else 0
        self.precision = precision
        self.handle = C.c_void_p()
        _lib.check(_lib.lib().acg_batch_create(data.handle, C.cast(arr, C.c_void_p), len(self.pats),
                                               C.byref(opt), _stream_ptr(stream),
                                               C.byref(self.handle)), "acg_batch_create")
        self.outs = None

    def run(self, outs=None, stream=None):
        """Match every pattern; returns (or fills) one [Dn][Pn_i] float64 tensor each.

        Reusing the same output tensors relaunches the captured CUDA graph."""
        torch = _torch()
        if outs is None:
            if self.outs is None:
                dev = self.data.dev.node_feats.device
                self.outs = [torch.empty((self.data.num_nodes, p.num_nodes), dtype=torch.float64,
                                         device=dev) for p in self.pats]
            outs = self.outs
        ptrs = (C.c_void_p * len(outs))(*[o.data_ptr() for o in outs])
        _lib.check(_lib.lib().acg_batch_match(self.handle, C.cast(ptrs, C.c_void_p),
                                              _stream_ptr(stream)), "acg_batch_match")
        return outs

    def info(self) -> dict:
        inf = _lib.BatchInfo()
        _lib.check(_lib.lib().acg_batch_get_info(self.handle, C.byref(inf)), "acg_batch_get_info")
        return {k: getattr(inf, k) for k, _ in _lib.BatchInfo._fields_}

    def close(self):
        if self.handle:
            _lib.lib().acg_batch_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
