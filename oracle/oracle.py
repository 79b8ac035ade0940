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
    """Build liboracle.so, and the reference CPU binary when its sources exist."""
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    ref = reference_dir or os.environ.get("ACG_REFERENCE_DIR", "/root/reference")
    if Path(ref, "src", "main.cu").exists():
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
