"""Adjoint kernels (Cholesky, triangular solve, log-determinant) and the GP
loss gradient, checked against central finite differences (h = 1e-6) and a
torch.linalg (CPU, float64) reference gradient.  The torch.autograd.Function
below exists only in this test harness."""
import numpy as np
import pytest
import torch

from mat_gb300.api import as_colmajor, colmajor

pytestmark = pytest.mark.gpu


def spd(n, seed):
    g = torch.Generator().manual_seed(seed)
    a = torch.randn(n, n, generator=g, dtype=torch.float64)
    return a @ a.T / n + torch.eye(n, dtype=torch.float64)


class GpuCholesky(torch.autograd.Function):
    """L = chol(A) through mg_dpotrf, backward through mg_dpotrf_backward."""

    @staticmethod
    def forward(ctx, A, handle):
        L = as_colmajor(A.detach().cuda())
        assert handle.dpotrf(L) == 0
        ctx.handle = handle
        ctx.save_for_backward(L)
        return L.cpu().clone()

    @staticmethod
    def backward(ctx, Lbar):
        (L,) = ctx.saved_tensors
        Ab = ctx.handle.dpotrf_backward(L, as_colmajor(torch.tril(Lbar).cuda()))
        return Ab.cpu().clone(), None


def test_cholesky_adjoint_matches_torch_and_fd(handle):
    n = 160
    A = spd(n, 1)
    g = torch.Generator().manual_seed(2)
    W = torch.tril(torch.randn(n, n, generator=g, dtype=torch.float64))
    # ours
    Ag = A.clone().requires_grad_(True)
    (GpuCholesky.apply(Ag, handle) * W).sum().backward()
    ours = Ag.grad
    # torch.linalg reference (symmetrised gradient)
    At = A.clone().requires_grad_(True)
    (torch.linalg.cholesky(At) * W).sum().backward()
    ref = 0.5 * (At.grad + At.grad.T)
    assert torch.allclose(ours, ours.T)
    assert (ours - ref).norm() / ref.norm() < 1e-10
    # central differences along a symmetric direction
    E = torch.randn(n, n, generator=g, dtype=torch.float64)
    E = 0.5 * (E + E.T)
    h = 1e-6
    f = lambda M: (torch.linalg.cholesky(M) * W).sum().item()
    fd = (f(A + h * E) - f(A - h * E)) / (2 * h)
    an = (ours * E).sum().item()
    assert abs(fd - an) / abs(an) < 1e-6


@pytest.mark.parametrize("trans", [False, True])
def test_trsm_adjoint(handle, trans):
    n, k = 130, 3
    A = spd(n, 3)
    L = torch.linalg.cholesky(A)
    g = torch.Generator().manual_seed(4)
    B = torch.randn(n, k, generator=g, dtype=torch.float64)
    Xbar = torch.randn(n, k, generator=g, dtype=torch.float64)
    # torch reference
    Lt = L.clone().requires_grad_(True)
    Bt = B.clone().requires_grad_(True)
    X = torch.linalg.solve_triangular(Lt.T if trans else Lt, Bt, upper=trans)
    (X * Xbar).sum().backward()
    # ours
    Ld = as_colmajor(L.cuda())
    Lbar = as_colmajor(torch.zeros(n, n, dtype=torch.float64).cuda())
    Bbar = handle.dtrsm_backward(Ld, as_colmajor(X.detach().cuda()), as_colmajor(Xbar.cuda()), Lbar, trans=trans)
    torch.cuda.synchronize()
    assert (Bbar.cpu() - Bt.grad).norm() / Bt.grad.norm() < 1e-12
    lb = torch.tril(Lbar.cpu())
    assert (lb - torch.tril(Lt.grad)).norm() / Lt.grad.norm() < 1e-12


def test_logdet_and_adjoint(handle):
    n = 90
    A = spd(n, 5)
    L = as_colmajor(torch.linalg.cholesky(A).cuda())
    ld = handle.dlogdet_chol(L)
    assert abs(ld - torch.logdet(A).item()) < 1e-12 * abs(ld) + 1e-12
    Lbar = as_colmajor(torch.zeros(n, n, dtype=torch.float64).cuda())
    handle.dlogdet_chol_backward(L, 0.5, Lbar)
    torch.cuda.synchronize()
    d = torch.diagonal(Lbar.cpu())
    assert torch.allclose(d, 1.0 / torch.diagonal(L.cpu()))


def gp_torch(Xp, y, ell, sigma2=1.0, jitter=1e-2):
    d2 = ((Xp[:, None, :] - Xp[None, :, :]) ** 2).sum(-1)
    K = sigma2 * torch.exp(-d2 / (2 * ell * ell)) + jitter * torch.eye(Xp.shape[0], dtype=Xp.dtype)
    L = torch.linalg.cholesky(K)
    z = torch.linalg.solve_triangular(L, y[:, None], upper=False)
    return 0.5 * (z * z).sum() + torch.log(torch.diagonal(L)).sum(), K


@pytest.mark.parametrize("n", [64, 257])
def test_gp_loss_gradient(handle, n):
    g = torch.Generator().manual_seed(6)
    Xp = torch.rand(n, 3, generator=g, dtype=torch.float64)
    y = torch.randn(n, generator=g, dtype=torch.float64)
    ell = 0.2
    loss, dell, Kb = handle.gp_loss_grad(as_colmajor(Xp.cuda()), y.cuda().contiguous(), ell, want_kbar=True)
    torch.cuda.synchronize()
    # torch.linalg reference gradient
    ellt = torch.tensor(ell, dtype=torch.float64, requires_grad=True)
    lt, K = gp_torch(Xp, y, ellt)
    K.retain_grad()
    lt.backward()
    assert abs(loss - lt.item()) < 1e-10 * abs(lt.item())
    assert abs(dell - ellt.grad.item()) < 1e-8 * abs(ellt.grad.item())
    kref = 0.5 * (K.grad + K.grad.T)
    assert (Kb.cpu() - kref).norm() / kref.norm() < 1e-9
    # closed form: dK = 0.5 (K^-1 - alpha alpha^T)
    Kd = K.detach()
    alpha = torch.linalg.solve(Kd, y)
    closed = 0.5 * (torch.linalg.inv(Kd) - torch.outer(alpha, alpha))
    assert (Kb.cpu() - closed).norm() / closed.norm() < 1e-8
    # central differences on the lengthscale, h = 1e-6
    h = 1e-6
    lp, _, _ = handle.gp_loss_grad(as_colmajor(Xp.cuda()), y.cuda().contiguous(), ell + h)
    lm, _, _ = handle.gp_loss_grad(as_colmajor(Xp.cuda()), y.cuda().contiguous(), ell - h)
    fd = (lp - lm) / (2 * h)
    assert abs(fd - dell) / abs(dell) < 1e-6
