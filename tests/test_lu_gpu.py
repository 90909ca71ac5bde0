"""Mat PLU / Solve_direct on the GPU against the oracle (the bit-identical
restatement of Mat-8.3.1's AVX-512 build): identical pivot permutation `pos`
and factors within 1e-13 normwise relative."""
import numpy as np
import pytest
import torch

from mat_gb300.api import as_colmajor, colmajor, host_fill_normal
from oracle.api import restatement

pytestmark = pytest.mark.gpu
TOL = 1e-13


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def gpu_plu(handle, a):
    A = as_colmajor(torch.from_numpy(a))
    pos, info = handle.dgetrf(A)
    torch.cuda.synchronize()
    lu = A.cpu().numpy()
    m, n = a.shape
    s = min(m, n)
    L = np.tril(lu[:, :s], -1) + np.eye(m, s)
    U = np.triu(lu[:s, :])
    return pos.cpu().numpy(), L, U, info


@pytest.mark.parametrize("n", [1, 2, 7, 61, 90, 91, 97, 120, 121, 180, 257, 1000])
def test_plu_square_matches_oracle(handle, n):
    a = host_fill_normal(n, n, seed=1)
    pos, L, U, info = gpu_plu(handle, a)
    assert info == 0
    opos, oL, oU = restatement().plu(a)
    assert np.array_equal(pos, opos), "pivot permutation differs from Mat's"
    assert rel(L, oL[:, :n]) < TOL and rel(U, oU[:n]) < TOL
    assert rel(a[pos], L @ U) < 1e-14 * max(1, n / 100)


@pytest.mark.parametrize("m,n", [(130, 61), (400, 250), (97, 96)])
def test_plu_tall_matches_oracle(handle, m, n):
    a = host_fill_normal(m, n, seed=2)
    pos, L, U, info = gpu_plu(handle, a)
    opos, oL, oU = restatement().plu(a)
    assert np.array_equal(pos, opos)
    assert rel(L, oL[:, :n]) < TOL and rel(U, oU[:n]) < TOL


def test_plu_ties_pick_first_row(handle):
    # integer-valued matrix with repeated magnitudes in every column: the
    # pivot must be the first row holding the largest |a| (Mat LU/__PLU.h:73-76)
    rng = np.random.default_rng(5)
    a = np.asfortranarray(rng.integers(-3, 4, size=(150, 150)).astype(np.float64))
    a += np.eye(150) * 0.0
    pos, L, U, info = gpu_plu(handle, a)
    opos, oL, oU = restatement().plu(a)
    assert info == 0 and np.array_equal(pos, opos)
    assert rel(U, oU[:150]) < TOL


def test_plu_singular_reports_column(handle):
    a = host_fill_normal(100, 100, seed=3)
    a[:, 37] = 0.0
    A = as_colmajor(torch.from_numpy(a))
    pos, info = handle.dgetrf(A)
    assert info == 38


@pytest.mark.parametrize("n,nrhs", [(1, 1), (50, 1), (300, 4), (1000, 1), (513, 3)])
def test_solve_narrow_matches_oracle(handle, n, nrhs):
    a = host_fill_normal(n, n, seed=1)
    b = host_fill_normal(n, nrhs, seed=2)
    X, info = handle.dgesv(as_colmajor(torch.from_numpy(a)), as_colmajor(torch.from_numpy(b)))
    torch.cuda.synchronize()
    x = X.cpu().numpy()
    ox = restatement().solve(a, b)
    assert info == 0
    assert rel(x, ox) < TOL * 10
    r = b - a @ x
    assert np.linalg.norm(r) / (np.linalg.norm(a) * np.linalg.norm(x)) < 1e-15


def test_getrs_reuses_factors(handle):
    n = 200
    a = host_fill_normal(n, n, seed=4)
    A = as_colmajor(torch.from_numpy(a))
    pos, info = handle.dgetrf(A)
    for seed in (5, 6):
        b = host_fill_normal(n, 2, seed=seed)
        X = handle.dgetrs(A, pos, as_colmajor(torch.from_numpy(b)))
        torch.cuda.synchronize()
        assert rel(X.cpu().numpy(), restatement().solve(a, b)) < 1e-12
