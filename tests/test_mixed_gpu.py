"""Mixed LU (fp32 panels + split-BF16 tensor-core updates) with FP64
iterative refinement: normwise backward error <= 1e-14 on Householder-product
matrices of condition 1e6, forward error against the plain FP64 GPU solve,
and the FP64 fallback when refinement stalls."""
import numpy as np
import pytest
import torch

from mat_gb300.api import colmajor

pytestmark = pytest.mark.gpu


def svd_matrix(handle, n, seed=3, sigma_min=1e-6, nrefl=64):
    A = colmajor(n, n)
    handle.gen_svd_matrix(A, seed, nrefl=nrefl, sigma_min=sigma_min)
    torch.cuda.synchronize()
    return A


def test_svd_generator_spectrum(handle):
    n = 300
    A = svd_matrix(handle, n, nrefl=16, sigma_min=1e-6).cpu().numpy()
    s = np.linalg.svd(A, compute_uv=False)
    expect = np.sort(1e-6 ** (np.arange(n) / (n - 1)))[::-1]
    assert np.allclose(s, expect, rtol=1e-8, atol=1e-14)


def backward_error(a, x, b):
    r = b - a @ x
    return (np.abs(r).max(0) / (np.abs(a).sum(1).max() * np.abs(x).max(0) + np.abs(b).max(0))).max()


@pytest.mark.parametrize("n,nrhs", [(300, 1), (1024, 4), (2500, 4), (1001, 3)])  # 1001: unaligned columns
def test_mixed_ir_reaches_fp64_backward_error(handle, n, nrhs):
    A = svd_matrix(handle, n)
    B = colmajor(n, nrhs)
    handle.fill_normal(B, 11)
    X, rep = handle.dsgesv_ir(A, B, tol=1e-14)
    torch.cuda.synchronize()
    assert rep["status"] == 0 and rep["path"] == 0, rep
    a, b, x = A.cpu().numpy(), B.cpu().numpy(), X.cpu().numpy()
    eta = backward_error(a, x, b)
    assert eta <= 1e-14, (eta, rep)
    # forward error against the plain FP64 GPU solve (both near cond * eps)
    Xd, info = handle.dgesv(A, B)
    xd = Xd.cpu().numpy()
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-7
    # pivot growth max|U| / max|A| of the fp32 factorization, as mg_sgetrf gives it
    A32 = A.float().t().contiguous().t()
    handle.sgetrf(A32)
    torch.cuda.synchronize()
    growth = float(torch.triu(A32).abs().max()) / float(A.abs().max())
    assert abs(rep["pivot_growth"] - growth) <= 1e-6 * growth, (rep["pivot_growth"], growth)


def test_mixed_ir_fallback_when_refinement_stalls(handle):
    # one bf16 term (8-bit products) cannot reach 1e-14 at condition 1e6:
    # plain refinement stalls; with GMRES-IR off the FP64 fallback takes over
    n = 512
    A = svd_matrix(handle, n)
    B = colmajor(n, 2)
    handle.fill_normal(B, 12)
    X, rep = handle.dsgesv_ir(A, B, nterms=1, max_iter=6, gmres=False)
    torch.cuda.synchronize()
    assert rep["status"] == 7 and rep["path"] == 2, rep  # MG_FALLBACK_USED, FP64 path
    a, b, x = A.cpu().numpy(), B.cpu().numpy(), X.cpu().numpy()
    assert backward_error(a, x, b) <= 1e-14
    # and with every takeover disabled it reports the stall instead
    X2, rep2 = handle.dsgesv_ir(A, B, nterms=1, max_iter=6, fallback=False, gmres=False)
    assert rep2["status"] == 6 and rep2["backward_error"] > 1e-14, rep2  # MG_IR_STALLED


@pytest.mark.parametrize("n,sigma_min", [(2048, 1e-9), (4096, 1e-9)])
def test_gmres_ir_beyond_plain_refinement(handle, n, sigma_min):
    """At condition 1e9 plain refinement with the fp32 factors stalls; GMRES-IR
    (FP64 GMRES preconditioned by the same factors) reaches 1e-14 and reports
    path 1, with no FP64 refactorization."""
    A = svd_matrix(handle, n, seed=7, sigma_min=sigma_min)
    B = colmajor(n, 4)
    handle.fill_normal(B, 13)
    a, b = A.cpu().numpy(), B.cpu().numpy()
    Xp, rp = handle.dsgesv_ir(A, B, fallback=False, gmres=False)
    torch.cuda.synchronize()
    assert rp["status"] == 6, rp  # plain refinement alone does not get there
    X, rep = handle.dsgesv_ir(A, B, fallback=False, gmres=True)
    torch.cuda.synchronize()
    assert rep["status"] == 7 and rep["path"] == 1 and rep["gmres_iterations"] > 0, rep
    eta = backward_error(a, X.cpu().numpy(), b)
    assert eta <= 1e-14, (eta, rep)
