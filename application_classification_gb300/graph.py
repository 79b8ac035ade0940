"""Host graphs: the reference's binary/CSV formats and the seeded generators.

A :class:`Graph` holds numpy arrays in the layout of ``struct Graph``
(src/main.cu:8-19): f64 ``node_feats[N][Kv]``, f64 ``edge_feats[M][Ke]``,
u64 ``srcs[M]``, u64 ``dsts[M]``.  File I/O and generation run in the native
library (``include/acg_io.h``); graphs it makes are zero-copy numpy views of
library memory, each view keeping that memory alive.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import _lib


@dataclass
class Graph:
    node_feats: np.ndarray  # [N][Kv] float64
    edge_feats: np.ndarray  # [M][Ke] float64
    srcs: np.ndarray  # [M] uint64
    dsts: np.ndarray  # [M] uint64
    meta: dict = field(default_factory=dict)
    _mem: object = field(default=None, repr=False, compare=False)

    def __post_init__(self):
        self.node_feats = np.ascontiguousarray(self.node_feats, dtype=np.float64)
        self.edge_feats = np.ascontiguousarray(self.edge_feats, dtype=np.float64)
        if self.node_feats.ndim != 2 or self.edge_feats.ndim != 2:
            raise ValueError("features must be 2-D")
        self.srcs = np.ascontiguousarray(self.srcs, dtype=np.uint64)
        self.dsts = np.ascontiguousarray(self.dsts, dtype=np.uint64)
        if not (len(self.srcs) == len(self.dsts) == self.edge_feats.shape[0]):
            raise ValueError("srcs, dsts and edge_feats disagree on the edge count")

    @property
    def num_nodes(self) -> int:
        return self.node_feats.shape[0]

    @property
    def num_edges(self) -> int:
        return self.edge_feats.shape[0]

    @property
    def node_feat_dim(self) -> int:
        return self.node_feats.shape[1]

    @property
    def edge_feat_dim(self) -> int:
        return self.edge_feats.shape[1]

    def nbytes(self) -> int:
        return sum(a.nbytes for a in (self.node_feats, self.edge_feats, self.srcs, self.dsts))

    # -------- C views
    def _host_struct(self) -> _lib.HostGraph:
        h = _lib.HostGraph()
        h.num_nodes, h.node_feat_dim = self.node_feats.shape
        h.num_edges, h.edge_feat_dim = self.edge_feats.shape
        h.node_feats = self.node_feats.ctypes.data_as(_lib.f64p)
        h.edge_feats = self.edge_feats.ctypes.data_as(_lib.f64p)
        h.srcs = self.srcs.ctypes.data_as(_lib.u64p)
        h.dsts = self.dsts.ctypes.data_as(_lib.u64p)
        return h

    def c_graph(self) -> _lib.Graph:
        """``acg_graph`` with HOST pointers into this object's arrays."""
        g = _lib.Graph()
        g.num_nodes, g.node_feat_dim = self.node_feats.shape
        g.num_edges, g.edge_feat_dim = self.edge_feats.shape
        g.node_feats = self.node_feats.ctypes.data
        g.edge_feats = self.edge_feats.ctypes.data
        g.srcs = self.srcs.ctypes.data
        g.dsts = self.dsts.ctypes.data
        return g

    # -------- files
    def write_bin(self, path) -> None:
        h = self._host_struct()
        _lib.check(_lib.lib().acg_graph_write_bin(str(path).encode(), C.byref(h)), "write_bin")

    def write_csv(self, vertex_csv, edges_csv) -> None:
        h = self._host_struct()
        e = str(edges_csv).encode() if edges_csv is not None else None
        _lib.check(_lib.lib().acg_graph_write_csv(str(vertex_csv).encode(), e, C.byref(h)),
                   "write_csv")

    @staticmethod
    def read_bin(path) -> "Graph":
        h = _lib.HostGraph()
        _lib.check(_lib.lib().acg_graph_read_bin(str(path).encode(), C.byref(h)), "read_bin")
        return _adopt(h)

    @staticmethod
    def read_csv(vertex_csv, edges_csv=None) -> "Graph":
        h = _lib.HostGraph()
        e = str(edges_csv).encode() if edges_csv is not None else None
        _lib.check(_lib.lib().acg_graph_read_csv(str(vertex_csv).encode(), e, C.byref(h)),
                   "read_csv")
        return _adopt(h)


class _HostMem:
    """Owns a library-allocated ``acg_host_graph``; frees it when collected."""

    def __init__(self, h: _lib.HostGraph):
        self.h = h

    def __del__(self):
        try:
            _lib.lib().acg_host_graph_free(C.byref(self.h))
        except Exception:
            pass


class _View:
    """Array interface over library memory that keeps its owner alive: every
    numpy view made from it holds a reference to the ``_HostMem``."""

    def __init__(self, mem: _HostMem, ptr, count: int, typestr: str):
        self.mem = mem
        addr = C.cast(ptr, C.c_void_p).value
        self.__array_interface__ = {"data": (addr, False), "shape": (count,),
                                    "typestr": typestr, "version": 3}


def _views(mem: _HostMem):
    h = mem.h
    n, kv, m, ke = h.num_nodes, h.node_feat_dim, h.num_edges, h.edge_feat_dim

    def arr(ptr, count, dtype):
        if count == 0:
            return np.zeros(0, dtype=dtype)
        return np.asarray(_View(mem, ptr, count, np.dtype(dtype).str))

    return (arr(h.node_feats, n * kv, np.float64).reshape(n, kv),
            arr(h.edge_feats, m * ke, np.float64).reshape(m, ke),
            arr(h.srcs, m, np.uint64), arr(h.dsts, m, np.uint64))


def _adopt(h: _lib.HostGraph) -> Graph:
    """Wrap a library-allocated graph as a Graph of zero-copy numpy views."""
    mem = _HostMem(h)
    g = Graph(*_views(mem))
    g._mem = mem
    return g


def _refresh(g: Graph) -> None:
    g.node_feats, g.edge_feats, g.srcs, g.dsts = _views(g._mem)


def _owned(g: Graph) -> Graph:
    """``g`` itself if its arrays are library memory, else a library-owned copy."""
    if getattr(g, "_mem", None) is not None:
        return g
    h = _lib.HostGraph()
    n, kv = g.node_feats.shape
    m, ke = g.edge_feats.shape
    _lib.check(_lib.lib().acg_host_graph_alloc(C.byref(h), n, kv, m, ke), "alloc")
    out = _adopt(h)
    out.node_feats[...] = g.node_feats
    out.edge_feats[...] = g.edge_feats
    out.srcs[...] = g.srcs
    out.dsts[...] = g.dsts
    out.meta = dict(g.meta)
    return out


# ------------------------------------------------------------------ generators
def gen_er(n: int, m: int, kv: int = 13, ke: int = 17, seed: int = 0) -> Graph:
    h = _lib.HostGraph()
    _lib.check(_lib.lib().acg_gen_er(n, m, kv, ke, seed, C.byref(h)), "gen_er")
    g = _adopt(h)
    g.meta.update(kind="er", n=n, m=m, seed=seed)
    return g


def gen_rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19,
             c: float = 0.19, kv: int = 13, ke: int = 17, seed: int = 0) -> Graph:
    h = _lib.HostGraph()
    _lib.check(_lib.lib().acg_gen_rmat(scale, edge_factor, a, b, c, kv, ke, seed, C.byref(h)),
               "gen_rmat")
    g = _adopt(h)
    g.meta.update(kind="rmat", scale=scale, edge_factor=edge_factor, seed=seed)
    return g


def plant(data: Graph, pn: int, pe: int, noise: float = 0.05, seed: int = 0):
    """Plant a pattern; returns ``(data2, pattern, truth_vertex, truth_edge)``.

    ``data2`` is ``data`` with any planted new edges appended: the same object,
    updated in place, when ``data`` holds library memory (any generated or
    file-read graph), else a library-owned copy."""
    d = _owned(data)
    tv = np.zeros(pn, dtype=np.uint64)
    te = np.zeros(pe, dtype=np.uint64)
    hp = _lib.HostGraph()
    st = _lib.lib().acg_gen_plant(C.byref(d._mem.h), pn, pe, noise, seed, C.byref(hp),
                                  tv.ctypes.data_as(_lib.u64p), te.ctypes.data_as(_lib.u64p))
    _refresh(d)
    _lib.check(st, "plant")
    p = _adopt(hp)
    p.meta.update(kind="planted", pn=pn, pe=pe, noise=noise, seed=seed)
    return d, p, tv, te[: p.num_edges]


def fill_edges(g: Graph, m: int, seed: int = 0) -> Graph:
    """Top ``g`` up with random new edges to exactly ``m`` edges (in place when
    ``g`` holds library memory)."""
    d = _owned(g)
    st = _lib.lib().acg_gen_fill_edges(C.byref(d._mem.h), m, seed)
    _refresh(d)
    _lib.check(st, "fill_edges")
    return d


# ------------------------------------------------------------------ workloads
def workload(name: str):
    """The synthetic workloads, by name: returns ``(data, pattern, truth_vertex)``.

    er1k      : Erdos-Renyi 1,000 vertices / 20,000 edges, pattern 10 / 20, seed 0
    rmat18    : R-MAT scale 18, edge factor 16, pattern 16 / 32, seed 1
    rmat22    : R-MAT scale 22, edge factor 16, pattern 32 / 64, seed 2
    rmat16    : R-MAT scale 16, pattern 12 / 24, seed 4
    rmat12    : R-MAT scale 12, pattern 12 / 24, seed 4
    rmatS_P_E : R-MAT scale S, pattern P vertices / E edges, seed S (tests)
    All features i.i.d. N(0,1) (13-dim vertex, 17-dim edge); pattern features
    are the planted elements' features plus N(0, 0.05^2) noise.
    """
    if name == "er1k":
        d = gen_er(1000, 20000 - 20, seed=0)
        d, p, tv, _ = plant(d, 10, 20, 0.05, seed=0)
        d = fill_edges(d, 20000, seed=0)
        return d, p, tv
    table = {"rmat18": (18, 16, 32, 1), "rmat22": (22, 32, 64, 2),
             "rmat16": (16, 12, 24, 4), "rmat12": (12, 12, 24, 4), "rmat20": (20, 16, 32, 3)}
    if name in table:
        s, pn, pe, seed = table[name]
    elif name.startswith("rmat") and name.count("_") == 2:
        a, b, c = name[4:].split("_")
        s, pn, pe, seed = int(a), int(b), int(c), int(a)
    else:
        raise KeyError(name)
    d = gen_rmat(s, 16, seed=seed)
    d, p, tv, _ = plant(d, pn, pe, 0.05, seed=seed)
    return d, p, tv


def batch_workload(scale: int = 20, npatterns: int = 64, seed: int = 3):
    """Many patterns of uneven size planted in one R-MAT graph.

    Data: R-MAT scale ``scale``, edge factor 16, seed ``seed``.  Pattern i:
    Pn uniform in 4..48, Pe uniform in 2 Pn..4 Pn (at most Pn (Pn - 1)), planted with seed
    1000 * seed + i (features + N(0, 0.05^2)).  Returns (data, patterns,
    truth_vertices)."""
    rng = np.random.default_rng(seed)
    d = gen_rmat(scale, 16, seed=seed)
    pats, truths = [], []
    for i in range(npatterns):
        pn = int(rng.integers(4, 49))
        pe = min(int(rng.integers(2 * pn, 4 * pn + 1)), pn * (pn - 1))  # distinct edges only
        d, p, tv, _ = plant(d, pn, pe, 0.05, seed=1000 * seed + i)
        pats.append(p)
        truths.append(tv)
    return d, pats, truths
