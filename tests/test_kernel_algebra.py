"""The restructured algebra of the kernels reproduces the reference (CPU only)."""
import numpy as np
import pytest

from conftest import golden_names, load_golden
import kernel_algebra


@pytest.mark.parametrize("name", golden_names())
def test_algebra_fp64_matches_reference(name):
    d, p, ref = load_golden(name)
    mu = kernel_algebra.match(d, p)
    assert np.abs(mu - ref).max() <= 1e-10 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("iters", [0, 1, 2])
def test_algebra_partial_iterations(iters):
    from oracle import oracle

    d, p, _ = load_golden("irregular")
    a = kernel_algebra.match(d, p, num_iters=iters)
    b = oracle.match(d, p, num_iters=iters)
    assert np.abs(a - b).max() <= 1e-10 * max(1.0, np.abs(b).max())


@pytest.mark.parametrize("name", ["er300", "rmat9", "georgiy"])
def test_cnull_oracle_vs_algebra(name):
    """The optional C-null term (test.py:93-97, left out by the reference): the
    oracle's pass-by-pass form and the restructured algebra agree, and the term
    changes the result on these graphs (it cancels only where a column's fill
    wins at every data vertex: then it shifts the whole column, which the
    column normaliser removes)."""
    from oracle import oracle

    d, p, ref = load_golden(name)
    a = kernel_algebra.match(d, p, cnull=True)
    b = oracle.match(d, p, cnull=True)
    assert np.abs(a - b).max() <= 1e-10 * max(1.0, np.abs(b).max())
    assert np.abs(b - ref).max() > 1e-6
