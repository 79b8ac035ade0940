"""TEST INFRASTRUCTURE: ctypes binding of the CPU oracle (oracle/acg_oracle.c).

The oracle restates the reference matcher (src/main.cu:66-257,
src/ac.hxx:17-186) in plain C, FP64, pass by pass.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg use it, always as the
checker or the CPU baseline -- never as the thing measured or shipped.
Also wraps the unmodified reference built for the CPU (oracle/_ref), which
exists only where the reference sources were available to build it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
REF_BIN = HERE / "_ref" / "ac_ref_omp"


class _OG(C.Structure):
    _fields_ = [("num_nodes", C.c_uint64), ("node_feat_dim", C.c_uint64),
                ("num_edges", C.c_uint64), ("edge_feat_dim", C.c_uint64),
                ("node_feats", C.c_void_p), ("edge_feats", C.c_void_p),
                ("srcs", C.c_void_p), ("dsts", C.c_void_p)]


_L = None


def build(reference_dir: str | None = None) -> None:
    """Build liboracle.so, and the reference CPU binary when a reference
    checkout is given (``reference_dir`` or the environment variable
    ACG_REFERENCE_DIR) and holds its sources."""
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    ref = reference_dir or os.environ.get("ACG_REFERENCE_DIR")
    if ref and Path(ref, "src", "main.cu").exists():
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF={ref}"], check=True,
                       stderr=subprocess.DEVNULL)


def lib():
    global _L
    if _L is None:
        if not LIB.exists():
            build()
        L = C.CDLL(str(LIB))
        L.acg_oracle_match.argtypes = [C.POINTER(_OG), C.POINTER(_OG), C.c_int64, C.c_void_p,
                                       C.POINTER(C.c_double)]
        L.acg_oracle_match.restype = C.c_int
        L.acg_oracle_match_opts.argtypes = [C.POINTER(_OG), C.POINTER(_OG), C.c_int64, C.c_int,
                                            C.c_void_p, C.POINTER(C.c_double)]
        L.acg_oracle_match_opts.restype = C.c_int
        L.acg_oracle_check.argtypes = [C.POINTER(_OG), C.POINTER(_OG)]
        L.acg_oracle_check.restype = C.c_int
        L.acg_oracle_threads.restype = C.c_int
        L.acg_oracle_set_threads.argtypes = [C.c_int]
        _L = L
    return _L


def _og(g) -> _OG:
    return _OG(g.num_nodes, g.node_feat_dim, g.num_edges, g.edge_feat_dim,
               g.node_feats.ctypes.data, g.edge_feats.ctypes.data,
               g.srcs.ctypes.data, g.dsts.ctypes.data)


def match(data, pattern, num_iters: int = -1, threads: int | None = None,
          return_elapsed: bool = False, cnull: bool = False):
    """Oracle mu [Dn][Pn] (float64) for host graphs (``graph.Graph``); ``cnull``
    adds the optional C-null term."""
    L = lib()
    if threads:
        L.acg_oracle_set_threads(int(threads))
    mu = np.zeros((data.num_nodes, pattern.num_nodes), dtype=np.float64)
    gd, gp = _og(data), _og(pattern)
    el = C.c_double(0.0)
    rc = L.acg_oracle_match_opts(C.byref(gd), C.byref(gp), int(num_iters), 1 if cnull else 0,
                                 mu.ctypes.data if mu.size else None, C.byref(el))
    if rc != 0:
        raise ValueError(f"oracle rejected the input (code {rc})")
    return (mu, el.value) if return_elapsed else mu


def reference_available() -> bool:
    return REF_BIN.exists()


def reference_match(data, pattern, threads: int | None = None, return_elapsed: bool = False):
    """Run the unmodified reference (CPU build) on host graphs; exact mu doubles."""
    if not REF_BIN.exists():
        raise FileNotFoundError(REF_BIN)
    with tempfile.TemporaryDirectory() as td:
        dp, pp, out = Path(td, "data.bin"), Path(td, "pattern.bin"), Path(td, "mu.bin")
        data.write_bin(dp)
        pattern.write_bin(pp)
        env = dict(os.environ, ACG_REF_BIN=str(out), ACG_REF_QUIET="1")
        if threads:
            env["OMP_NUM_THREADS"] = str(threads)
        r = subprocess.run([str(REF_BIN), str(dp), str(pp)], env=env, capture_output=True,
                           text=True, check=True)
        mu = np.fromfile(out, dtype=np.float64).reshape(data.num_nodes, pattern.num_nodes)
        elapsed = None
        for line in r.stderr.splitlines():
            if line.startswith("elapsed="):
                elapsed = float(line.split("=", 1)[1])
    return (mu, elapsed) if return_elapsed else mu


# ------------------------------------------------------------------ workloads
# Seeded synthetic graphs made by the oracle's own generator
# (oracle/acg_oracle_gen.c): the same bytes as the product's generator for the
# same arguments, without loading the product library.  The CPU baseline and
# the reference arm of the benchmark build their workloads with these.

class _AG(C.Structure):
    _fields_ = [("num_nodes", C.c_uint64), ("node_feat_dim", C.c_uint64),
                ("num_edges", C.c_uint64), ("edge_feat_dim", C.c_uint64),
                ("node_feats", C.c_void_p), ("edge_feats", C.c_void_p),
                ("srcs", C.c_void_p), ("dsts", C.c_void_p)]


class OGraph:
    """A host graph (numpy arrays in the layout of ``struct Graph``, main.cu:8-19)."""

    def __init__(self, node_feats, edge_feats, srcs, dsts):
        self.node_feats = np.ascontiguousarray(node_feats, dtype=np.float64)
        self.edge_feats = np.ascontiguousarray(edge_feats, dtype=np.float64)
        self.srcs = np.ascontiguousarray(srcs, dtype=np.uint64)
        self.dsts = np.ascontiguousarray(dsts, dtype=np.uint64)

    num_nodes = property(lambda self: self.node_feats.shape[0])
    node_feat_dim = property(lambda self: self.node_feats.shape[1])
    num_edges = property(lambda self: self.edge_feats.shape[0])
    edge_feat_dim = property(lambda self: self.edge_feats.shape[1])

    def write_bin(self, path) -> None:
        """The reference's binary graph layout (main.cu:21-44, prob2bin.py:42-62)."""
        with open(path, "wb") as f:
            np.array([self.num_nodes, self.node_feat_dim, self.num_edges, self.edge_feat_dim],
                     dtype=np.uint64).tofile(f)
            for a in (self.node_feats, self.edge_feats, self.srcs, self.dsts):
                a.tofile(f)


def _gen_lib():
    L = lib()
    if not hasattr(L, "_gen_ready"):
        P = C.POINTER(_AG)
        L.acgo_gen_rmat.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                    C.c_uint64, C.c_uint64, C.c_uint64, P]
        L.acgo_gen_er.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint64, P]
        L.acgo_fill_edges.argtypes = [P, C.c_uint64, C.c_uint64]
        L.acgo_plant.argtypes = [P, C.c_uint64, C.c_uint64, C.c_double, C.c_uint64, P, C.c_void_p,
                                 C.c_void_p]
        L.acgo_free.argtypes = [P]
        for f in (L.acgo_gen_rmat, L.acgo_gen_er, L.acgo_fill_edges, L.acgo_plant):
            f.restype = C.c_int
        L.acgo_free.restype = None
        L._gen_ready = True
    return L


def _adopt(h: _AG) -> OGraph:
    """Copy a library-made graph into numpy arrays and free it."""
    n, kv, m, ke = h.num_nodes, h.node_feat_dim, h.num_edges, h.edge_feat_dim

    def arr(ptr, count, ctype, dtype):
        if count == 0:
            return np.zeros(0, dtype=dtype)
        return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ctype)), shape=(count,)).copy()

    g = OGraph(arr(h.node_feats, n * kv, C.c_double, np.float64).reshape(n, kv),
               arr(h.edge_feats, m * ke, C.c_double, np.float64).reshape(m, ke),
               arr(h.srcs, m, C.c_uint64, np.uint64), arr(h.dsts, m, C.c_uint64, np.uint64))
    _gen_lib().acgo_free(C.byref(h))
    return g


def _to_c(g: OGraph) -> _AG:
    """A C copy of an OGraph (malloc'd arrays, which the C side may reallocate)."""
    libc = C.CDLL(None)
    libc.malloc.restype = C.c_void_p
    libc.malloc.argtypes = [C.c_size_t]
    h = _AG(g.num_nodes, g.node_feat_dim, g.num_edges, g.edge_feat_dim, None, None, None, None)
    for name, a in (("node_feats", g.node_feats), ("edge_feats", g.edge_feats), ("srcs", g.srcs),
                    ("dsts", g.dsts)):
        p = libc.malloc(max(1, a.nbytes))
        if not p:
            raise MemoryError
        if a.nbytes:
            C.memmove(p, a.ctypes.data, a.nbytes)
        setattr(h, name, p)
    return h


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise ValueError(f"{what}: code {rc}")


def gen_rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19,
             c: float = 0.19, kv: int = 13, ke: int = 17, seed: int = 0) -> OGraph:
    h = _AG()
    _check(_gen_lib().acgo_gen_rmat(scale, edge_factor, a, b, c, kv, ke, seed, C.byref(h)), "gen_rmat")
    return _adopt(h)


def gen_er(n: int, m: int, kv: int = 13, ke: int = 17, seed: int = 0) -> OGraph:
    h = _AG()
    _check(_gen_lib().acgo_gen_er(n, m, kv, ke, seed, C.byref(h)), "gen_er")
    return _adopt(h)


def fill_edges(g: OGraph, m: int, seed: int = 0) -> OGraph:
    h = _to_c(g)
    rc = _gen_lib().acgo_fill_edges(C.byref(h), m, seed)
    out = _adopt(h)
    _check(rc, "fill_edges")
    return out


def plant(data: OGraph, pn: int, pe: int, noise: float = 0.05, seed: int = 0):
    """Returns (data with any new edges appended, pattern, truth_vertex, truth_edge)."""
    h = _to_c(data)
    hp = _AG()
    tv = np.zeros(pn, dtype=np.uint64)
    te = np.zeros(pe, dtype=np.uint64)
    rc = _gen_lib().acgo_plant(C.byref(h), pn, pe, noise, seed, C.byref(hp), tv.ctypes.data,
                               te.ctypes.data)
    d = _adopt(h)
    _check(rc, "plant")
    p = _adopt(hp)
    return d, p, tv, te[: p.num_edges]


def workload(name: str):
    """The named synthetic workloads (the same graphs as the product's
    ``graph.workload``): returns ``(data, pattern, truth_vertex)``."""
    if name == "er1k":
        d = gen_er(1000, 20000 - 20, seed=0)
        d, p, tv, _ = plant(d, 10, 20, 0.05, seed=0)
        return fill_edges(d, 20000, seed=0), p, tv
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
