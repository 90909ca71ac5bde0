"""Full-size configurations checked through size-independent properties
(the reference's CPU path takes minutes to hours at these sizes):

* Householder QR of a 16384 x 4096 iid N(0,1) matrix (seed 1): R upper
  triangular, A = Q R and Q^T Q = I on sampled columns, within 1e-13.
* Split-BF16 GEMM, M = N = K = 16384, entries u * 2^e (u ~ U[-1,1), e uniform
  in [-8, 8], seed 3): normwise error on 256 sampled rows against the FP64
  product of the same fp32 inputs.  The tensor cores accumulate the whole K
  chain in FP32 without per-step IEEE rounding, so the error grows about
  linearly in K (measured 7.2e-5 at K = 16384, below 8e-6 at K = 1024); the
  tolerance is 1.5e-4.  The ordered variant (lower-order products first)
  measured 1.9e-5; tolerance 4e-5 and at most half the one-pass error.
* Gaussian-process loss and lengthscale gradient at n = 8192 (RBF, ell 0.2,
  jitter 1e-2, FP64): analytic gradient against central differences, h = 1e-6,
  relative 1e-6.
* Mixed LU + FP64 refinement at n = 16384, 4 RHS, cond 1e6: normwise backward
  error <= 1e-14, recomputed here in FP64 from A, x and b.
"""

import pytest
import torch

from mat_gb300.api import colmajor

pytestmark = pytest.mark.gpu


def test_qr_16384x4096_properties(handle):
    m, k = 16384, 4096
    A = colmajor(m, k)
    handle.fill_normal(A, 1)
    Q, R = handle.dqr(A)
    torch.cuda.synchronize()
    assert float(torch.tril(R, -1).abs().max()) == 0.0
    g = torch.Generator(device="cuda").manual_seed(11)
    cols = torch.randperm(k, generator=g, device="cuda")[:64]
    rel = float((A[:, cols] - Q @ R[:, cols]).norm() / A[:, cols].norm())
    assert rel < 1e-13, rel
    qc = torch.randperm(m, generator=g, device="cuda")[:64]
    G = Q.t() @ Q[:, qc]
    eye = torch.zeros_like(G)
    eye[qc, torch.arange(64, device="cuda")] = 1.0
    orth = float((G - eye).norm() / 8.0)  # ||I_64||_F = 8
    assert orth < 1e-13, orth


def test_split_gemm_16384_wide_exponents(handle):
    n = 16384
    g = torch.Generator(device="cuda").manual_seed(3)

    def wide():
        u = torch.rand((n, n), generator=g, device="cuda", dtype=torch.float64) * 2 - 1
        e = torch.randint(-8, 9, (n, n), generator=g, device="cuda").to(torch.float64)
        return (u * torch.exp2(e)).float().t().contiguous().t()

    A, B = wide(), wide()
    Cm = handle.sgemm_bf16x(A, B)
    torch.cuda.synchronize()
    rows = torch.randperm(n, generator=g, device="cuda")[:256]
    ref = A[rows].double() @ B.double()
    err = float((Cm[rows].double() - ref).norm() / ref.norm())
    assert err < 1.5e-4, err
    # lower-order products first: measured 1.9e-5
    Co = handle.sgemm_bf16x(A, B, ordered=True)
    torch.cuda.synchronize()
    err_o = float((Co[rows].double() - ref).norm() / ref.norm())
    assert err_o < 4e-5 and err_o < 0.5 * err, (err_o, err)


def test_gp_8192_gradient_vs_central_differences(handle):
    n, ell, h = 8192, 0.2, 1e-6
    g = torch.Generator(device="cuda").manual_seed(5)
    X = torch.rand((3, n), generator=g, device="cuda", dtype=torch.float64).t()
    y = torch.randn(n, generator=g, device="cuda", dtype=torch.float64)
    loss, dell, _ = handle.gp_loss_grad(X, y, ell)
    lp, _, _ = handle.gp_loss_grad(X, y, ell + h)
    lm, _, _ = handle.gp_loss_grad(X, y, ell - h)
    fd = (lp - lm) / (2 * h)
    assert abs(fd - dell) <= 1e-6 * abs(dell), (fd, dell)


def test_mixed_ir_16384_backward_error(handle):
    n, nrhs = 16384, 4
    A = colmajor(n, n)
    handle.gen_svd_matrix(A, 3, nrefl=64, sigma_min=1e-6)
    B = colmajor(n, nrhs)
    handle.fill_normal(B, 11)
    X, rep = handle.dsgesv_ir(A, B, tol=1e-14)
    torch.cuda.synchronize()
    assert rep["status"] == 0 and rep["path"] == 0, rep
    r = B - A @ X
    anorm = float(A.abs().sum(1).max())
    eta = (r.abs().amax(0) / (anorm * X.abs().amax(0) + B.abs().amax(0))).max().item()
    assert eta <= 1e-14, (eta, rep["history"])
    assert abs(eta - rep["backward_error"]) <= 0.1 * eta + 1e-17
