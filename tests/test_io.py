"""Host I/O of the reference's front end, on the CPU: the binary graph format
(loadGraph, src/main.cu:21-44; prob2bin.py:42-62), the CSV pair layout
(prob2bin.py:11-40), the native converter that replaces prob2bin.py, and the
mu writers (printf("%e\\n") per entry, src/main.cu:255-257)."""
import ctypes as C
import subprocess

import numpy as np
import pytest

from conftest import load_golden
from application_classification_gb300 import _lib, build, graph
from application_classification_gb300._lib import AcgError

TOOLS = build.BUILD


def _same(a, b):
    assert (a.num_nodes, a.node_feat_dim, a.num_edges, a.edge_feat_dim) == \
           (b.num_nodes, b.node_feat_dim, b.num_edges, b.edge_feat_dim)
    for x, y in ((a.node_feats, b.node_feats), (a.edge_feats, b.edge_feats),
                 (a.srcs, b.srcs), (a.dsts, b.dsts)):
        assert np.array_equal(np.asarray(x), np.asarray(y))


def test_bin_round_trip_is_byte_exact(tmp_path):
    d, _, _ = load_golden("er300")
    p = tmp_path / "g.bin"
    d.write_bin(p)
    _same(graph.Graph.read_bin(p), d)
    g = graph.gen_er(50, 200, seed=3)
    g.write_bin(p)
    _same(graph.Graph.read_bin(p), g)


def test_bin_layout_matches_prob2bin(tmp_path):
    g = graph.gen_er(7, 11, kv=3, ke=2, seed=1)
    p = tmp_path / "g.bin"
    g.write_bin(p)
    raw = p.read_bytes()
    hdr = np.frombuffer(raw[:32], dtype=np.uint64)
    assert list(hdr) == [7, 3, 11, 2]
    off = 32
    nf = np.frombuffer(raw[off:off + 7 * 3 * 8], dtype=np.float64); off += 7 * 3 * 8
    ef = np.frombuffer(raw[off:off + 11 * 2 * 8], dtype=np.float64); off += 11 * 2 * 8
    s = np.frombuffer(raw[off:off + 11 * 8], dtype=np.uint64); off += 11 * 8
    t = np.frombuffer(raw[off:off + 11 * 8], dtype=np.uint64); off += 11 * 8
    assert off == len(raw)
    assert np.array_equal(nf, np.asarray(g.node_feats).ravel())
    assert np.array_equal(ef, np.asarray(g.edge_feats).ravel())
    assert np.array_equal(s, np.asarray(g.srcs)) and np.array_equal(t, np.asarray(g.dsts))


def test_bin_truncated_is_an_io_error(tmp_path):
    d, _, _ = load_golden("tiny")
    p = tmp_path / "g.bin"
    d.write_bin(p)
    raw = p.read_bytes()
    for cut in (0, 16, len(raw) - 8):
        p.write_bytes(raw[:cut])
        with pytest.raises(AcgError) as e:
            graph.Graph.read_bin(p)
        assert e.value.status == 6  # ACG_ERR_IO


def test_csv_round_trip(tmp_path):
    g = graph.gen_rmat(8, 4, seed=5)
    v, e = tmp_path / "g.Vertex.csv", tmp_path / "g.Edges.csv"
    g.write_csv(v, e)
    _same(graph.Graph.read_csv(v, e), g)


def test_csv_reference_layout(tmp_path):
    # header "N C" then "id f..." / "src dst f...", space separated
    v, e = tmp_path / "p.Vertex.csv", tmp_path / "p.Edges.csv"
    v.write_text("3 3\n0 0.5 -1\n1 2 3.25\n2 1e-3 -4\n")
    e.write_text("2 3\n0 1 7.5\n2 0 -0.125\n")
    g = graph.Graph.read_csv(v, e)
    assert (g.num_nodes, g.node_feat_dim, g.num_edges, g.edge_feat_dim) == (3, 2, 2, 1)
    assert np.array_equal(np.asarray(g.node_feats), [[0.5, -1], [2, 3.25], [1e-3, -4]])
    assert np.array_equal(np.asarray(g.edge_feats), [[7.5], [-0.125]])
    assert list(np.asarray(g.srcs)) == [0, 2] and list(np.asarray(g.dsts)) == [1, 0]


def test_csv_vertex_ids_must_be_row_numbers(tmp_path):
    v = tmp_path / "p.Vertex.csv"
    v.write_text("2 2\n0 1.0\n5 2.0\n")  # prob2bin.py:28-29 asserts id == row
    with pytest.raises(AcgError):
        graph.Graph.read_csv(v, None)


def test_prob2bin_tool(tmp_path):
    d, _, _ = load_golden("er300")
    src = tmp_path / "d.bin"
    d.write_bin(src)
    v, e, out = tmp_path / "d.Vertex.csv", tmp_path / "d.Edges.csv", tmp_path / "d2.bin"
    tool = str(TOOLS / "acg_prob2bin")
    subprocess.run([tool, "--to-csv", str(src), str(v), str(e)], check=True, capture_output=True)
    subprocess.run([tool, str(v), str(e), str(out)], check=True, capture_output=True)
    assert out.read_bytes() == src.read_bytes()
    assert subprocess.run([tool], capture_output=True).returncode == 2
    assert subprocess.run([tool, str(tmp_path / "missing.csv"), str(e), str(out)],
                          capture_output=True).returncode == 1


def test_mu_text_matches_printf_e(tmp_path):
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.normal(0, 50, 3000), rng.normal(0, 1e-6, 500),
                        [0.0, -0.0, 1e300, -1e-300, np.inf, -np.inf, 5e-324, 0.5, 9.9999995e-7]])
    mu = np.ascontiguousarray(x.reshape(-1, 1))
    p = tmp_path / "mu.txt"
    _lib.check(_lib.lib().acg_mu_write_text(str(p).encode(), mu.ctypes.data, mu.shape[0], 1), "write")
    assert p.read_text() == "".join("%e\n" % v for v in x)


def test_mu_text_to_stdout_and_bin(tmp_path):
    mu = np.arange(12, dtype=np.float64).reshape(4, 3) / 7
    code = ("import sys, numpy as np; sys.path.insert(0, %r); "
            "from application_classification_gb300 import _lib; "
            "mu = np.arange(12, dtype=np.float64).reshape(4, 3) / 7; "
            "_lib.lib().acg_mu_write_text(None, mu.ctypes.data, 4, 3)") % str(build.ROOT)
    r = subprocess.run(["python", "-c", code], capture_output=True, text=True, check=True)
    assert r.stdout == "".join("%e\n" % v for v in mu.ravel())
    p = tmp_path / "mu.bin"
    _lib.check(_lib.lib().acg_mu_write_bin(str(p).encode(), mu.ctypes.data, 4, 3), "write")
    assert np.array_equal(np.fromfile(p, dtype=np.float64).reshape(4, 3), mu)


def test_driver_usage_errors():
    exe = str(TOOLS / "acg_main")
    assert subprocess.run([exe], capture_output=True).returncode == 2
    assert subprocess.run([exe, "--precision", "fp16", "a", "b"], capture_output=True).returncode == 2
    r = subprocess.run([exe, "/nonexistent/d.bin", "/nonexistent/p.bin"], capture_output=True, text=True)
    assert r.returncode == 1 and "nonexistent" in r.stderr
