"""The native host driver (drop-in for the reference program) on the GPU: its
"%e" text equals the match to print precision, its binary output equals the
C-ABI match, and the CSV front end gives the same result."""
import subprocess

import numpy as np
import pytest

from conftest import load_golden
from application_classification_gb300 import build

pytestmark = pytest.mark.gpu

EXE = str(build.BUILD / "acg_main")
FP64_REL = 1e-10


def _golden_paths(tmp_path, name):
    d, p, ref = load_golden(name)
    dp, pp = tmp_path / "data.bin", tmp_path / "pattern.bin"
    d.write_bin(dp)
    p.write_bin(pp)
    return d, p, ref, dp, pp


def test_driver_text_output(cuda, tmp_path):
    d, p, ref, dp, pp = _golden_paths(tmp_path, "er300")
    r = subprocess.run([EXE, str(dp), str(pp)], capture_output=True, text=True, check=True)
    assert r.stderr.startswith("elapsed=")
    mu = np.array([float(x) for x in r.stdout.split()]).reshape(d.num_nodes, p.num_nodes)
    # "%e" keeps 7 significant digits
    assert np.all(np.abs(mu - ref) <= 5e-7 * np.abs(ref) + 1e-300)


def test_driver_binary_output_and_csv_front_end(cuda, tmp_path):
    d, p, ref, dp, pp = _golden_paths(tmp_path, "rmat9")
    out = tmp_path / "mu.bin"
    subprocess.run([EXE, "--binary", "--out", str(out), str(dp), str(pp)], check=True,
                   capture_output=True)
    mu = np.fromfile(out, dtype=np.float64).reshape(d.num_nodes, p.num_nodes)
    assert np.abs(mu - ref).max() <= FP64_REL * max(1.0, np.abs(ref).max())
    d.write_csv(tmp_path / "d.Vertex.csv", tmp_path / "d.Edges.csv")
    p.write_csv(tmp_path / "p.Vertex.csv", tmp_path / "p.Edges.csv")
    out2 = tmp_path / "mu2.bin"
    subprocess.run([EXE, "--csv", "--binary", "--out", str(out2), str(tmp_path / "d"),
                    str(tmp_path / "p")], check=True, capture_output=True)
    assert np.array_equal(np.fromfile(out2, dtype=np.float64), mu.ravel())


def test_driver_mixed_precision(cuda, tmp_path):
    d, p, ref, dp, pp = _golden_paths(tmp_path, "er300")
    out = tmp_path / "mu.bin"
    subprocess.run([EXE, "--precision", "mixed", "--binary", "--out", str(out), str(dp), str(pp)],
                   check=True, capture_output=True)
    mu = np.fromfile(out, dtype=np.float64).reshape(d.num_nodes, p.num_nodes)
    assert np.abs(mu - ref).max() <= 1e-4


def test_match_graphs_host_equals_device_path(cuda):
    """acg_match_graphs_host (host buffers in and out, the feature copies
    overlapped with the CSR build) gives the device path's mu bit for bit."""
    from application_classification_gb300 import graph, matcher

    d, p, _ = graph.workload("rmat10_9_18")
    for prec in ("fp64", "mixed"):
        a = matcher.match_host(d, p, prec)
        b = matcher.match(d, p, prec)
        assert np.array_equal(a, b), prec


@pytest.mark.parametrize("dn,de,ke,pn,pe", [(50, 9, 17, 3, 2), (300, 3001, 17, 6, 10), (2000, 20003, 3, 8, 16),
                                            (1000, 9000, 40, 5, 8), (500, 4000, 13, 20, 70),
                                            (500, 4000, 32, 30, 100)])
def test_match_graphs_host_pieces(cuda, dn, de, ke, pn, pe):
    """Mixed precision: the one-shot call uploads the edge features in 16
    pieces and builds each piece's FP32 rows and edge-cost rows as it lands
    (rows scattered into destination-CSR order).  Same bits as the device path
    for piece sizes of 0 rows and ragged ones, a feature dim past the
    tensor-core limit (FP32 rows only), a pattern past 64 columns, and one whose
    cost matrix takes the chained tensor-core kernel (rows through its row map)."""
    from application_classification_gb300 import graph, matcher

    d = graph.gen_er(dn, de - pe, kv=13, ke=ke, seed=dn + de)
    d, p, _, _ = graph.plant(d, pn, pe, 0.05, seed=ke)
    a = matcher.match_host(d, p, "mixed")
    b = matcher.match(d, p, "mixed")
    assert np.array_equal(a, b)
    # the C-null term (it reads the edge cost matrix the pieces wrote)
    a = matcher.match_host(d, p, "mixed", cnull=True)
    b = matcher.match(d, p, "mixed", cnull=True)
    assert np.array_equal(a, b)


def test_release_cached_memory(cuda):
    """Objects freed to the library's pool can be handed back to the driver;
    matching works again afterwards."""
    import torch
    from application_classification_gb300 import _lib, graph, matcher

    d, p, _ = graph.workload("rmat10_9_18")
    first = matcher.match(d, p, "mixed")
    _lib.check(_lib.lib().acg_release_cached_memory(), "acg_release_cached_memory")
    free_after, _ = torch.cuda.mem_get_info()
    again = matcher.match(d, p, "mixed")
    assert np.array_equal(first, again)
    assert free_after > 0


def test_plain_allocator_gives_identical_output(cuda, tmp_path):
    """ACG_MEMPOOL=0 (plain cudaMalloc instead of the stream-ordered pool)
    changes where buffers live, not what is computed: the bytes are equal."""
    import os

    d, p, ref, dp, pp = _golden_paths(tmp_path, "rmat9")
    outs = []
    for flag in ("1", "0"):
        out = tmp_path / f"mu{flag}.bin"
        env = dict(os.environ, ACG_MEMPOOL=flag)
        subprocess.run([EXE, "--precision", "mixed", "--binary", "--out", str(out), str(dp),
                        str(pp)], check=True, capture_output=True, env=env)
        outs.append(out.read_bytes())
    assert outs[0] == outs[1]
