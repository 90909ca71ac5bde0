"""The seeded benchmark inputs as the oracle regenerates them on the host
(oracle.api.host_fill_*, gen_svd_matrix), checked against the library's own
host fills bit for bit and against the mathematics of the Q1 diag(sigma) Q2
recipe.  (The GPU generator is compared with the oracle's in
tests/test_inputs_gpu.py.)"""
import numpy as np
import pytest

from mat_gb300.api import host_fill_normal as lib_normal
from mat_gb300.api import host_fill_uniform as lib_uniform
from oracle.api import gen_svd_matrix, host_fill_normal, host_fill_uniform


@pytest.mark.parametrize("rows,cols,seed", [(1, 1, 0), (7, 5, 3), (300, 200, 1), (1000, 4, 11), (513, 300, 7)])
@pytest.mark.parametrize("rowmajor", [True, False])
def test_oracle_fills_equal_library_fills(rows, cols, seed, rowmajor):
    assert np.array_equal(host_fill_normal(rows, cols, seed, rowmajor), lib_normal(rows, cols, seed, rowmajor))
    assert np.array_equal(host_fill_uniform(rows, cols, seed, -1.0, 1.0, rowmajor),
                          lib_uniform(rows, cols, seed, -1.0, 1.0, rowmajor))


@pytest.mark.parametrize("n,smin", [(1, 1e-6), (2, 1e-6), (257, 1e-6), (4096, 1e-6), (100, 1e-12), (50, 1.0)])
def test_geometric_sigma(n, smin):
    """With no reflectors A = diag(sigma), sigma_r = smin^(r/(n-1)) from the
    generator's own exp / log series: within 1e-14 relative of numpy's power
    (the rounding of log(smin), scaled by up to |log smin|, sets that),
    sigma_0 = 1 exactly, strictly decreasing."""
    a = gen_svd_matrix(n, 3, 0, smin)
    s = np.diag(a)
    assert np.count_nonzero(a - np.diag(s)) == 0
    assert s[0] == 1.0
    if n > 1:
        ref = smin ** (np.arange(n) / (n - 1))
        assert np.all(np.abs(s - ref) <= 1e-14 * ref)
        if smin < 1.0:
            assert np.all(np.diff(s) < 0)


def test_svd_matrix_spectrum():
    """Q1, Q2 orthogonal: the singular values are sigma (to rounding), cond 1e6."""
    n = 300
    a = gen_svd_matrix(n, 5, 64, 1e-6)
    sv = np.linalg.svd(a, compute_uv=False)
    ref = 1e-6 ** (np.arange(n) / (n - 1))
    assert np.allclose(sv, ref, rtol=1e-9, atol=1e-15)
    assert gen_svd_matrix(n, 5, 64, 1e-6).tobytes() == a.tobytes()  # deterministic, thread count aside


@pytest.mark.parametrize("smin", [0.0, -1.0, 2.0])
def test_svd_matrix_rejects_bad_sigma(smin):
    with pytest.raises(ValueError):
        gen_svd_matrix(10, 1, 4, smin)
