"""Regenerate the golden fixtures in this folder (TEST INFRASTRUCTURE).

Each case is a (data.bin, pattern.bin) pair in the reference's binary format
plus mu.bin: the exact doubles that the UNMODIFIED reference program
(src/main.cu of porumbes/application_classification, built for the CPU with
Thrust's OpenMP backend by oracle/Makefile's `ref` target, output captured in
binary by oracle/ref_shim) prints for that pair.  Needs a checkout of the
reference sources, named by the environment variable ACG_REFERENCE_DIR:

    ACG_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from application_classification_gb300 import build as _build  # noqa: E402
from application_classification_gb300.graph import Graph, gen_er, gen_rmat, plant  # noqa: E402
from oracle import oracle  # noqa: E402

_ref = os.environ.get("ACG_REFERENCE_DIR")
if not _ref:
    raise SystemExit("set ACG_REFERENCE_DIR to the reference checkout")
REF = Path(_ref)


def georgiy():
    """The reference's own shipped fixtures (data/georgiy*.csv: data vertices,
    pattern vertices and pattern edges) plus synthetic data edges, since
    data/georgiyData.Edges.csv is not in the reference snapshot."""
    rng = np.random.default_rng(7)
    dv = Graph.read_csv(REF / "data/georgiyData.Vertex.csv")
    pat = Graph.read_csv(REF / "data/georgiyPattern.Vertex.csv", REF / "data/georgiyPattern.Edges.csv")
    n, m = dv.num_nodes, 4000
    src = rng.integers(0, n, m)
    dst = (src + rng.integers(1, n, m)) % n
    pick = rng.integers(0, pat.num_edges, m)
    ef = pat.edge_feats[pick] + rng.normal(0.0, 2.0, (m, pat.edge_feat_dim))
    data = Graph(dv.node_feats, ef, src.astype(np.uint64), dst.astype(np.uint64))
    return data, pat


def er300():
    d = gen_er(300, 2990, seed=11)
    d, p, _, _ = plant(d, 6, 10, 0.05, seed=11)
    return d, p


def rmat9():
    d = gen_rmat(9, 8, seed=9)
    d, p, _, _ = plant(d, 8, 16, 0.05, seed=9)
    return d, p


def irregular():
    """Multi-edges, self-loops, isolated vertices, a hub whose in- and out-degree
    exceed the 256-edge chunk, a pattern with a self-loop and a repeated edge."""
    rng = np.random.default_rng(5)
    n = 200
    src = list(rng.integers(0, 150, 900))  # vertices 150..199 mostly isolated
    dst = list(rng.integers(0, 150, 900))
    src += [3] * 600 + list(rng.integers(0, 150, 600))  # hub 3: out-degree > 600
    dst += list(rng.integers(0, 150, 600)) + [7] * 600  # hub 7: in-degree > 600
    src += [10, 10, 10, 20, 20]  # multi-edges and self-loops
    dst += [11, 11, 10, 20, 21]
    m = len(src)
    data = Graph(rng.normal(size=(n, 13)), rng.normal(size=(m, 17)),
                 np.array(src, dtype=np.uint64), np.array(dst, dtype=np.uint64))
    ps = np.array([0, 1, 2, 3, 4, 2, 1, 1], dtype=np.uint64)
    pd = np.array([1, 2, 3, 4, 0, 2, 2, 2], dtype=np.uint64)
    pv = data.node_feats[[3, 7, 10, 20, 11]] + rng.normal(0, 0.05, (5, 13))
    pe = rng.normal(size=(8, 17))
    return data, Graph(pv, pe, ps, pd)


def tiny():
    rng = np.random.default_rng(1)
    data = Graph(rng.normal(size=(3, 4)), rng.normal(size=(4, 3)),
                 np.array([0, 1, 2, 0], np.uint64), np.array([1, 2, 0, 2], np.uint64))
    pat = Graph(rng.normal(size=(2, 4)), rng.normal(size=(2, 3)),
                np.array([0, 1], np.uint64), np.array([1, 0], np.uint64))
    return data, pat


def small_data():
    """A pattern larger than the data graph (9 vertices / 12 edges against 5 /
    8, with self-loops on both sides); Pn*Dn = 45 < Pe*De = 96, so the
    reference's quirk negation stays inside its buffers."""
    rng = np.random.default_rng(13)
    ds = np.array([0, 1, 2, 3, 4, 1, 2, 0], np.uint64)
    dd = np.array([1, 2, 3, 4, 0, 3, 2, 4], np.uint64)
    data = Graph(rng.normal(size=(5, 13)), rng.normal(size=(8, 17)), ds, dd)
    ps = np.array([i for i in range(9)] + [0, 2, 8], np.uint64)
    pd = np.array([(i + 1) % 9 for i in range(9)] + [5, 7, 8], np.uint64)
    return data, Graph(rng.normal(size=(9, 13)), rng.normal(size=(12, 17)), ps, pd)


def one_data_vertex():
    """One data vertex with two parallel self-loops; a 3-vertex path pattern."""
    rng = np.random.default_rng(17)
    data = Graph(rng.normal(size=(1, 13)), rng.normal(size=(2, 17)),
                 np.array([0, 0], np.uint64), np.array([0, 0], np.uint64))
    pat = Graph(rng.normal(size=(3, 13)), rng.normal(size=(2, 17)),
                np.array([0, 1], np.uint64), np.array([1, 2], np.uint64))
    return data, pat


CASES = {"georgiy": georgiy, "er300": er300, "rmat9": rmat9, "irregular": irregular, "tiny": tiny,
         "small_data": small_data, "one_data_vertex": one_data_vertex}


def main(names=None):
    """Regenerate the named cases (all when none are named); the manifest keeps
    the entries of the others."""
    _build.build()
    oracle.build(str(REF))
    mpath = HERE / "manifest.json"
    manifest = json.loads(mpath.read_text()) if mpath.exists() else {}
    for name, fn in CASES.items():
        if names and name not in names:
            continue
        d, p = fn()
        out = HERE / name
        out.mkdir(exist_ok=True)
        d.write_bin(out / "data.bin")
        p.write_bin(out / "pattern.bin")
        mu = oracle.reference_match(d, p)
        mu.tofile(out / "mu.bin")
        manifest[name] = {
            "data": [d.num_nodes, d.node_feat_dim, d.num_edges, d.edge_feat_dim],
            "pattern": [p.num_nodes, p.node_feat_dim, p.num_edges, p.edge_feat_dim],
            "mu_md5": hashlib.md5(mu.tobytes()).hexdigest(),
            "max_abs_mu": float(np.abs(mu).max()),
        }
        print(name, manifest[name])
    manifest = {k: manifest[k] for k in CASES if k in manifest}
    mpath.write_text(json.dumps(manifest, indent=1) + "\n")


if __name__ == "__main__":
    main(sys.argv[1:])
