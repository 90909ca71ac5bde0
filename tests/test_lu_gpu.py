"""Mat PLU / Solve_direct / Inv on the GPU against the oracle (the
bit-identical restatement of Mat-8.3.1's AVX-512 build): identical pivot
permutation `pos`, factors within 1e-13 normwise relative, solves and
inverses bit for bit."""
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


@pytest.mark.parametrize(
    "n,nrhs",
    [(1, 1), (50, 1), (300, 4), (1000, 1), (513, 3),  # narrow path
     (5, 5), (80, 9), (90, 16), (91, 8), (121, 17), (600, 7), (700, 145), (1031, 300)],  # wide path
)
def test_solve_matches_oracle(handle, n, nrhs):
    """Bit-identical to Mat's Solve_direct on both of its paths (the oracle is
    pinned to the reference build on every shape the reference runs)."""
    a = host_fill_normal(n, n, seed=1)
    b = host_fill_normal(n, nrhs, seed=2)
    X, info = handle.dgesv(as_colmajor(torch.from_numpy(a)), as_colmajor(torch.from_numpy(b)))
    torch.cuda.synchronize()
    x = X.cpu().numpy()
    ox = restatement().solve(a, b)
    assert info == 0
    assert np.array_equal(x, ox)
    r = b - a @ x
    assert np.linalg.norm(r) / (np.linalg.norm(a) * np.linalg.norm(x)) < 1e-15


def test_getrs_reuses_factors(handle):
    n = 200
    a = host_fill_normal(n, n, seed=4)
    A = as_colmajor(torch.from_numpy(a))
    pos, info = handle.dgetrf(A)
    for seed, k in ((5, 2), (6, 2), (7, 12)):
        b = host_fill_normal(n, k, seed=seed)
        X = handle.dgetrs(A, pos, as_colmajor(torch.from_numpy(b)))
        torch.cuda.synchronize()
        assert np.array_equal(X.cpu().numpy(), restatement().solve(a, b))


@pytest.mark.parametrize("n", [1, 2, 8, 9, 17, 60, 89, 90, 91, 150, 181, 517])
def test_inv_matches_oracle(handle, n):
    """Mat's Inv bit for bit: one block for n <= 90, blocks of 60 above."""
    a = host_fill_normal(n, n, seed=21)
    X, info = handle.dinv(as_colmajor(torch.from_numpy(a)))
    torch.cuda.synchronize()
    assert info == 0
    assert np.array_equal(X.cpu().numpy(), restatement().inv(a))


def test_inv_in_place_and_strided(handle):
    n = 130
    a = host_fill_normal(n, n, seed=22)
    big = colmajor(n + 7, n)  # A is a view with leading dimension n + 7
    big[:n].copy_(torch.from_numpy(a))
    A = big[:n]
    X, info = handle.dinv(A, A)
    torch.cuda.synchronize()
    assert info == 0 and np.array_equal(A.cpu().numpy(), restatement().inv(a))


@pytest.mark.parametrize("n", [1, 2, 60, 89, 90, 91, 150, 517])
@pytest.mark.parametrize("dominant", [True, False])
def test_lu_without_pivoting_matches_oracle(handle, n, dominant):
    """Mat's LU (no interchanges) bit for bit, on diagonally dominant and on
    plain N(0,1) matrices (no zero pivots at these seeds)."""
    a = host_fill_normal(n, n, seed=4)
    if dominant:
        a[np.diag_indices(n)] += n
    A = as_colmajor(torch.from_numpy(a))
    info = handle.dlu(A)
    torch.cuda.synchronize()
    f = A.cpu().numpy()
    L0, U0 = restatement().lu(a)
    assert info == 0
    assert np.array_equal(np.tril(f, -1) + np.eye(n), L0) and np.array_equal(np.triu(f), U0)


def test_lu_without_pivoting_zero_pivot(handle):
    a = host_fill_normal(100, 100, seed=5)
    a[0, 0] = 0.0
    A = as_colmajor(torch.from_numpy(a))
    assert handle.dlu(A) == 1
