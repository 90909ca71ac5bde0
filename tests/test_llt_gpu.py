"""Mat LLT (blocked Cholesky) and LDLT on the GPU against the oracle
(bit-identical restatement of Mat-8.3.1's AVX-512 build); Cholesky factors
within 1e-13 normwise relative, LDLT bit for bit, non-SPD / zero-pivot
detection, and the Cholesky solve."""
import numpy as np
import pytest
import torch

from mat_gb300.api import as_colmajor, colmajor, host_fill_normal
from oracle.api import restatement

pytestmark = pytest.mark.gpu
TOL = 1e-13


def spd(n, seed=1):
    g = host_fill_normal(n, n, seed)
    return np.asfortranarray(g @ g.T / n + np.eye(n))


@pytest.mark.parametrize("n", [1, 2, 47, 48, 49, 96, 97, 145, 300, 1000])
def test_llt_matches_oracle(handle, n):
    s = spd(n)
    A = as_colmajor(torch.from_numpy(s))
    info = handle.dpotrf(A)
    torch.cuda.synchronize()
    L = A.cpu().numpy()
    ref = restatement().llt(s)
    assert info == 0
    assert np.linalg.norm(L - ref) / np.linalg.norm(ref) < TOL
    assert np.array_equal(np.triu(L, 1), np.zeros_like(L))
    assert np.linalg.norm(s - L @ L.T) / np.linalg.norm(s) < 1e-14


def test_llt_reads_lower_triangle_only(handle):
    s = spd(130, 2)
    garbage = s.copy(order="F")
    garbage[np.triu_indices(130, 1)] = 1e300
    A = as_colmajor(torch.from_numpy(garbage))
    handle.dpotrf(A)
    assert np.linalg.norm(A.cpu().numpy() - restatement().llt(s)) / np.linalg.norm(s) < TOL


def test_llt_not_spd_reports_column(handle):
    s = spd(120, 3)
    s[70, 70] = -5.0
    A = as_colmajor(torch.from_numpy(s))
    info = handle.dpotrf(A)
    assert info > 0 and info <= 71


@pytest.mark.parametrize("n,nrhs", [(5, 1), (200, 3), (1000, 4)])
def test_cholesky_solve(handle, n, nrhs):
    s = spd(n, 4)
    b = host_fill_normal(n, nrhs, 5)
    L = as_colmajor(torch.from_numpy(s))
    assert handle.dpotrf(L) == 0
    X = as_colmajor(torch.from_numpy(b))
    handle.dpotrs(L, X)
    torch.cuda.synchronize()
    x = X.cpu().numpy()
    assert np.linalg.norm(s @ x - b) / (np.linalg.norm(s) * np.linalg.norm(x)) < 1e-15


def sym(n, seed=3):
    g = host_fill_normal(n, n, seed)
    return np.asfortranarray(g + g.T)


@pytest.mark.parametrize("n", [1, 2, 47, 48, 96, 97, 145, 300, 1000])
@pytest.mark.parametrize("kind", ["spd", "indefinite"])
def test_ldlt_bit_identical(handle, n, kind):
    """Mat's LDLT (no pivoting) bit for bit: L (with Mat's d (1/d) diagonal) and d."""
    a = spd(n) if kind == "spd" else sym(n)
    A = as_colmajor(torch.from_numpy(a))
    d, info = handle.dldlt(A)
    torch.cuda.synchronize()
    L0, D0 = restatement().ldlt(a)
    assert info == 0
    assert np.array_equal(A.cpu().numpy(), L0)
    assert np.array_equal(d.cpu().numpy(), np.diag(D0))


def test_ldlt_reads_lower_triangle_only(handle):
    a = sym(130)
    junk = a.copy()
    junk[np.triu_indices(130, 1)] = np.nan
    A = as_colmajor(torch.from_numpy(np.asfortranarray(junk)))
    d, info = handle.dldlt(A)
    torch.cuda.synchronize()
    L0, D0 = restatement().ldlt(a)
    assert np.array_equal(A.cpu().numpy(), L0) and np.array_equal(d.cpu().numpy(), np.diag(D0))


def test_ldlt_zero_pivot_reports_column(handle):
    a = sym(60)
    a[0, :] = 0.0
    a[:, 0] = 0.0
    A = as_colmajor(torch.from_numpy(np.asfortranarray(a)))
    d, info = handle.dldlt(A)
    assert info == 1
