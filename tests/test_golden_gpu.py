"""GPU results against the reference's own outputs (golden digests produced
by tests/golden/make_golden.py from Mat-8.3.1): the FP64 GEMM, PLU, Solve
(narrow and wide), LU without pivoting, LLT, LDLT, QR (blocked and
unblocked), Det and Inv reproduce Mat's AVX-512 results bit for bit, so the SHA-256
of the raw column-major output equals the reference's, at the benchmark
sizes (GEMM M=N=K=1024, PLU / LLT n = 8192)."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest
import torch

from mat_gb300.api import as_colmajor, colmajor, host_fill_normal

pytestmark = pytest.mark.gpu
G = Path(__file__).resolve().parent / "golden"
META = json.loads((G / "golden.json").read_text())["cases"]


def sha(a):
    return hashlib.sha256(np.asfortranarray(a).tobytes(order="F")).hexdigest()


def test_gemm_1024(handle):
    A, B = colmajor(1024, 1024), colmajor(1024, 1024)
    handle.fill_uniform(A, 0)
    handle.fill_uniform(B, 1)
    C = handle.dgemm(A, B)
    torch.cuda.synchronize()
    assert sha(C.cpu().numpy()) == META["gemm_1024"]["sha256"]


@pytest.mark.parametrize("n", [257, 1000, 8192])
def test_plu(handle, n):
    A = colmajor(n, n)
    handle.fill_normal(A, 1)
    pos, info = handle.dgetrf(A)
    torch.cuda.synchronize()
    assert np.array_equal(pos.cpu().numpy(), np.load(G / f"plu_{n}_pos.npy"))
    lu = A.cpu().numpy()
    L = np.tril(lu, -1) + np.eye(n)
    U = np.triu(lu)
    assert sha(L) == META[f"plu_{n}"]["sha256_L"]
    assert sha(U) == META[f"plu_{n}"]["sha256_U"]


@pytest.mark.parametrize("n,k", [(300, 4), (2048, 1), (50, 9), (300, 8), (300, 13), (1000, 150), (8192, 16)])
def test_solve(handle, n, k):
    A, B = colmajor(n, n), colmajor(n, k)
    handle.fill_normal(A, 1)
    handle.fill_normal(B, 2)
    X, info = handle.dgesv(A, B)
    torch.cuda.synchronize()
    assert sha(X.cpu().numpy()) == META[f"solve_{n}_{k}"]["sha256"]


@pytest.mark.parametrize("n", [300, 8192])
def test_llt(handle, n):
    S = colmajor(n, n)
    handle.gen_spd_gram(S, 1)
    assert handle.dpotrf(S) == 0
    torch.cuda.synchronize()
    assert sha(S.cpu().numpy()) == META[f"llt_{n}"]["sha256"]


@pytest.mark.parametrize("m,n", [(300, 200), (1000, 500)])
def test_qr(handle, m, n):
    A = colmajor(m, n)
    handle.fill_normal(A, 7)
    Q, R = handle.dqr(A)
    torch.cuda.synchronize()
    assert sha(R.cpu().numpy()) == META[f"qr_{m}x{n}"]["sha256_R"]
    assert sha(Q.cpu().numpy()) == META[f"qr_{m}x{n}"]["sha256_Q"]


def test_qr_unblocked_60x40_full_arrays(handle):
    # Mat's unblocked path (min(m, n) <= 96): Q and R as the reference returns them, bit for bit
    f = np.load(G / "qr_60x40.npz")
    A = as_colmajor(torch.from_numpy(host_fill_normal(60, 40, 7)))
    Q, R = handle.dqr(A)
    torch.cuda.synchronize()
    assert np.array_equal(Q.cpu().numpy(), f["Q"]) and np.array_equal(R.cpu().numpy(), f["R"])


def test_det_150(handle):
    A = as_colmajor(torch.from_numpy(host_fill_normal(150, 150, 5)))
    assert handle.ddet(A) == META["det_150"]["value"]


def test_inv_61_full_array(handle):
    A = as_colmajor(torch.from_numpy(host_fill_normal(61, 61, 9)))
    X, info = handle.dinv(A)
    torch.cuda.synchronize()
    assert info == 0 and np.array_equal(X.cpu().numpy(), np.load(G / "inv_61.npz")["X"])


@pytest.mark.parametrize("n", [97, 300, 1000, 2048])
def test_inv(handle, n):
    A = colmajor(n, n)
    handle.fill_normal(A, 9)
    X, info = handle.dinv(A)
    torch.cuda.synchronize()
    assert info == 0 and sha(X.cpu().numpy()) == META[f"inv_{n}"]["sha256"]


def sym(n, seed):
    g = host_fill_normal(n, n, seed)
    return np.asfortranarray(g + g.T)


def test_ldlt_90_full_arrays(handle):
    f = np.load(G / "ldlt_90.npz")
    A = as_colmajor(torch.from_numpy(sym(90, 3)))
    d, info = handle.dldlt(A)
    torch.cuda.synchronize()
    assert np.array_equal(A.cpu().numpy(), f["L"]) and np.array_equal(d.cpu().numpy(), f["d"])


@pytest.mark.parametrize("n", [97, 300, 1000])
def test_ldlt(handle, n):
    A = as_colmajor(torch.from_numpy(sym(n, 3)))
    d, info = handle.dldlt(A)
    torch.cuda.synchronize()
    assert sha(A.cpu().numpy()) == META[f"ldlt_{n}"]["sha256_L"]
    assert sha(d.cpu().numpy()[:, None]) == META[f"ldlt_{n}"]["sha256_d"]


def test_ldlt_spd_2048(handle):
    S = colmajor(2048, 2048)
    handle.gen_spd_gram(S, 1)
    d, info = handle.dldlt(S)
    torch.cuda.synchronize()
    assert info == 0
    assert sha(S.cpu().numpy()) == META["ldlt_spd_2048"]["sha256_L"]
    assert sha(d.cpu().numpy()[:, None]) == META["ldlt_spd_2048"]["sha256_d"]


def dd(n, seed=4):
    g = host_fill_normal(n, n, seed)
    g[np.diag_indices(n)] += n
    return np.asfortranarray(g)


def lu_factors(A):
    f = A.cpu().numpy()
    return np.tril(f, -1) + np.eye(f.shape[0]), np.triu(f)


def test_lu_90_full_arrays(handle):
    f = np.load(G / "lu_90.npz")
    A = as_colmajor(torch.from_numpy(dd(90)))
    assert handle.dlu(A) == 0
    L, U = lu_factors(A)
    assert np.array_equal(L, f["L"]) and np.array_equal(U, f["U"])


@pytest.mark.parametrize("n", [300, 1000])
def test_lu(handle, n):
    A = as_colmajor(torch.from_numpy(dd(n)))
    assert handle.dlu(A) == 0
    L, U = lu_factors(A)
    assert sha(L) == META[f"lu_{n}"]["sha256_L"] and sha(U) == META[f"lu_{n}"]["sha256_U"]


# ------------------------------------------- the benchmark configurations
# Digests of the reference's own results at the benchmark sizes (make_golden.py
# --large; the single-threaded reference takes about five minutes for them).

def test_solve_8192_1_benchmark(handle):
    """The FP64 solve benchmark: A, b iid N(0,1) (seeds 1, 2), n = 8192, 1 RHS."""
    A, B = colmajor(8192, 8192), colmajor(8192, 1)
    handle.fill_normal(A, 1)
    handle.fill_normal(B, 2)
    X, info = handle.dgesv(A, B)
    torch.cuda.synchronize()
    assert sha(X.cpu().numpy()) == META["solve_8192_1"]["sha256"]


def test_solve_16384_4_benchmark(handle):
    """The FP64 side of the mixed-solve benchmark: its system (A = Q1 diag(sigma) Q2,
    seed 3, cond 1e6; B seed 11), solved by the FP64 GPU path bit for bit as
    Mat's Solve_direct solves it."""
    n = 16384
    A, B = colmajor(n, n), colmajor(n, 4)
    handle.gen_svd_matrix(A, 3, nrefl=64, sigma_min=1e-6)
    handle.fill_normal(B, 11)
    X, info = handle.dgesv(A, B)
    torch.cuda.synchronize()
    assert sha(X.cpu().numpy()) == META["solve_svd_16384_4"]["sha256"]


def test_qr_16384x4096_benchmark(handle):
    """The Householder QR benchmark with Mat's full 16384 x 16384 Q, bit for bit."""
    m, k = 16384, 4096
    A = colmajor(m, k)
    handle.fill_normal(A, 1)
    Q, R = handle.dqr(A)
    torch.cuda.synchronize()
    assert sha(R.cpu().numpy()) == META["qr_16384x4096"]["sha256_R"]
    assert sha(Q.cpu().numpy()) == META["qr_16384x4096"]["sha256_Q"]
