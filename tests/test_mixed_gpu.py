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
    # refinement stalls and the solve falls back to the FP64 path
    n = 512
    A = svd_matrix(handle, n)
    B = colmajor(n, 2)
    handle.fill_normal(B, 12)
    X, rep = handle.dsgesv_ir(A, B, nterms=1, max_iter=6)
    torch.cuda.synchronize()
    a, b, x = A.cpu().numpy(), B.cpu().numpy(), X.cpu().numpy()
    assert backward_error(a, x, b) <= 1e-14
    if rep["path"] == 2:
        assert rep["status"] == 7  # MG_FALLBACK_USED
    # and with the fallback disabled it reports the stall instead
    X2, rep2 = handle.dsgesv_ir(A, B, nterms=1, max_iter=2, fallback=False)
    assert rep2["status"] in (0, 6)
