"""ctypes declarations of the C ABI in ``include/acg.h`` and ``include/acg_io.h``.

The library is loaded from the package's ``_build/libacg.so`` (or from the
path in the environment variable ``ACG_LIBRARY``, a variant built by
``build.build(out_dir=...)``).  There is no fallback: if the library is
missing, :func:`lib` raises, so that nothing can silently run on another code
path.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

from . import build as _build

u64 = C.c_uint64
i32 = C.c_int32
i64 = C.c_int64
f64p = C.POINTER(C.c_double)
u64p = C.POINTER(C.c_uint64)
vp = C.c_void_p

ACG_OK = 0
STATUS_NAMES = {
    0: "ACG_OK",
    1: "ACG_ERR_INVALID_ARGUMENT",
    2: "ACG_ERR_OUT_OF_MEMORY",
    3: "ACG_ERR_INDEX_OUT_OF_RANGE",
    4: "ACG_ERR_CUDA",
    5: "ACG_ERR_UNSUPPORTED",
    6: "ACG_ERR_IO",
    7: "ACG_ERR_DEVICE_TIMEOUT",
}

PREC_FP64 = 0
PREC_MIXED = 1


class Graph(C.Structure):
    """``acg_graph``: mirrors ``struct Graph`` (src/main.cu:8-19)."""

    _fields_ = [
        ("num_nodes", u64),
        ("node_feat_dim", u64),
        ("num_edges", u64),
        ("edge_feat_dim", u64),
        ("node_feats", vp),
        ("edge_feats", vp),
        ("srcs", vp),
        ("dsts", vp),
    ]


class HostGraph(C.Structure):
    """``acg_host_graph``: host arrays owned by the library's allocator."""

    _fields_ = [
        ("num_nodes", u64),
        ("node_feat_dim", u64),
        ("num_edges", u64),
        ("edge_feat_dim", u64),
        ("node_feats", f64p),
        ("edge_feats", f64p),
        ("srcs", u64p),
        ("dsts", u64p),
        ("edge_capacity", u64),
    ]


class Options(C.Structure):
    _fields_ = [("precision", i32), ("num_iters", i32), ("kernel_timing", i32),
                ("edge_blocks_per_sm", i32), ("vertex_blocks_per_sm", i32),
                ("cnull", i32), ("cdist_kernel", i32), ("autotune", i32),
                ("edge_kernel", i32)]


class Stats(C.Structure):
    _fields_ = [
        ("ms_total", C.c_double),
        ("ms_cdist", C.c_double),
        ("ms_init", C.c_double),
        ("ms_iters", C.c_double),
        ("bytes_iters", C.c_double),
        ("bytes_edge_phase", C.c_double),
        ("bytes_vertex_phase", C.c_double),
        ("ms_edge_phase", C.c_double),
        ("ms_vertex_phase", C.c_double),
        ("launches", i64),
        ("num_iters", i64),
        ("edge_warps", i64),
        ("edge_ranges", i64),
        ("edge_heavy_vertices", i64),
    ]


class BatchInfo(C.Structure):
    _fields_ = [("patterns", i32), ("groups", i32), ("widest_group_columns", i32),
                ("autotuned", i32), ("graph_nodes", i64), ("ms_last", C.c_double),
                ("iter_ms_per_column", C.c_double), ("iter_ms_fixed", C.c_double),
                ("once_ms_per_column", C.c_double), ("once_ms_fixed", C.c_double),
                ("predicted_ms", C.c_double), ("edge_blocks_per_sm", i32),
                ("vertex_blocks_per_sm", i32)]


class AcgError(RuntimeError):
    """A C-ABI call returned a non-zero acg_status."""

    def __init__(self, status: int, where: str, message: str):
        self.status = status
        self.where = where
        self.message = message
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)}: {message}")


_P = C.POINTER
# name -> (restype, argtypes); every symbol the headers declare.
SIGNATURES: dict[str, tuple] = {
    # acg.h
    "acg_options_default": (None, [_P(Options)]),
    "acg_data_create": (i32, [_P(Graph), vp, _P(vp)]),
    "acg_data_destroy": (i32, [vp]),
    "acg_plan_create": (i32, [vp, _P(Graph), _P(Options), vp, _P(vp)]),
    "acg_plan_destroy": (i32, [vp]),
    "acg_match": (i32, [vp, vp, vp]),
    "acg_plan_stats": (i32, [vp, _P(Stats)]),
    "acg_match_graphs": (i32, [_P(Graph), _P(Graph), _P(Options), vp, vp]),
    "acg_match_graphs_host": (i32, [_P(Graph), _P(Graph), _P(Options), vp, vp]),
    "acg_release_cached_memory": (i32, []),
    "acg_inject_alloc_failure": (i32, [i64]),
    "acg_device_memory_in_use": (i32, [_P(i64)]),
    "acg_initial_mu_noalloc": (i32, [vp, u64, u64, vp, u64, vp, vp]),
    "acg_batch_create": (i32, [vp, vp, i32, _P(Options), vp, _P(vp)]),
    "acg_batch_match": (i32, [vp, vp, vp]),
    "acg_batch_get_info": (i32, [vp, _P(BatchInfo)]),
    "acg_batch_destroy": (i32, [vp]),
    "acg_match_record": (i32, [vp, vp, i32, vp]),
    "acg_backward": (i32, [vp, vp, vp, vp, vp, vp, vp]),
    "acg_status_string": (C.c_char_p, [i32]),
    "acg_last_error": (C.c_char_p, []),
    "acg_version": (C.c_char_p, []),
    # acg_io.h
    "acg_host_graph_alloc": (i32, [_P(HostGraph), u64, u64, u64, u64]),
    "acg_host_graph_free": (None, [_P(HostGraph)]),
    "acg_host_graph_view": (Graph, [_P(HostGraph)]),
    "acg_graph_read_bin": (i32, [C.c_char_p, _P(HostGraph)]),
    "acg_graph_write_bin": (i32, [C.c_char_p, _P(HostGraph)]),
    "acg_graph_read_csv": (i32, [C.c_char_p, C.c_char_p, _P(HostGraph)]),
    "acg_graph_write_csv": (i32, [C.c_char_p, C.c_char_p, _P(HostGraph)]),
    "acg_gen_er": (i32, [u64, u64, u64, u64, u64, _P(HostGraph)]),
    "acg_gen_rmat": (i32, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, u64, u64, u64,
                           _P(HostGraph)]),
    "acg_gen_plant": (i32, [_P(HostGraph), u64, u64, C.c_double, u64, _P(HostGraph), u64p, u64p]),
    "acg_gen_fill_edges": (i32, [_P(HostGraph), u64, u64]),
    "acg_mu_write_text": (i32, [C.c_char_p, vp, u64, u64]),
    "acg_mu_write_bin": (i32, [C.c_char_p, vp, u64, u64]),
}

_LIB: C.CDLL | None = None


def lib_path() -> Path:
    env = os.environ.get("ACG_LIBRARY")
    return Path(env) if env else _build.LIB


def lib() -> C.CDLL:
    """Load ``libacg.so`` (raise if it was not built)."""
    global _LIB
    if _LIB is None:
        p = lib_path()
        if not p.exists():
            raise RuntimeError(
                f"{p} is missing: build the native library first "
                "(python -m application_classification_gb300.build)")
        L = C.CDLL(str(p))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def check(status: int, where: str) -> None:
    if status != ACG_OK:
        msg = lib().acg_last_error().decode(errors="replace")
        raise AcgError(status, where, msg)
