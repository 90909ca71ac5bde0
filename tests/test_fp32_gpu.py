"""FP32 forms (Mat's templates on MAT<float>, the Gaussian-process workload run in FP32):
mg_sgemm against the FP64 product of the same fp32 inputs (normwise, 2e-6
scaled by sqrt(k/64) for the fp32 accumulation); mg_spotrf against the FP64
Cholesky of the same matrix; the FP32 Cholesky adjoint and the FP32
Gaussian-process gradient against their FP64 forms on the same fp32-exact
inputs.  FP32 carries the conditioning of K: at n = 8192 (cond(K) ~ 1e5) the
loss and gradient agree with FP64 to a few 1e-2 relative, which is the
tolerance used there."""
import pytest
import torch

from mat_gb300.api import as_colmajor, colmajor

pytestmark = pytest.mark.gpu


def rnd(m, n, seed, dtype=torch.float32):
    g = torch.Generator(device="cuda").manual_seed(seed)
    return (torch.rand((n, m), generator=g, device="cuda", dtype=torch.float64) * 2 - 1).to(dtype).t()


@pytest.mark.parametrize("m,n,k", [(1, 1, 1), (128, 128, 8), (200, 300, 70), (129, 257, 33), (1000, 130, 48),
                                   (512, 768, 1024)])
@pytest.mark.parametrize("ta,tb", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_sgemm(handle, m, n, k, ta, tb):
    A = rnd(k, m, 1) if ta else rnd(m, k, 1)
    B = rnd(n, k, 2) if tb else rnd(k, n, 2)
    C0 = rnd(m, n, 3)
    Cg = C0.clone()
    handle.sgemm(A, B, Cg, alpha=-1.0, beta=1.0, transA=bool(ta), transB=bool(tb))
    torch.cuda.synchronize()
    opA = A.double().t() if ta else A.double()
    opB = B.double().t() if tb else B.double()
    ref = C0.double() - opA @ opB
    err = float((Cg.double() - ref).norm() / ref.norm())
    assert err < 2e-6 * max(1.0, (k / 64) ** 0.5), err


def spd(n, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    G = torch.randn((n, n), generator=g, device="cuda", dtype=torch.float64)
    S = (G @ G.t() / n + torch.eye(n, device="cuda", dtype=torch.float64)).float().double()
    return S


@pytest.mark.parametrize("n", [1, 47, 96, 97, 300, 1000])
def test_spotrf(handle, n):
    S = spd(n, n)
    A = as_colmajor(S, dtype=torch.float32)
    assert handle.spotrf(A) == 0
    torch.cuda.synchronize()
    L = A.double()
    assert float(torch.triu(L, 1).abs().max()) == 0.0 if n > 1 else True
    ref = torch.linalg.cholesky(S)
    assert float((L - ref).norm() / ref.norm()) < 1e-5


def test_spotrf_not_spd(handle):
    S = spd(200, 1)
    S[150, 150] = -1.0
    A = as_colmajor(S, dtype=torch.float32)
    info = handle.spotrf(A)
    assert info >= 1


def test_spotrf_backward_matches_fp64(handle):
    n = 257
    S = spd(n, 7)
    L64 = torch.linalg.cholesky(S).float().double()
    g = torch.Generator(device="cuda").manual_seed(8)
    Lb64 = torch.tril(torch.randn((n, n), generator=g, device="cuda", dtype=torch.float64)).float().double()
    ref = handle.dpotrf_backward(as_colmajor(L64), as_colmajor(Lb64))
    got = handle.spotrf_backward(as_colmajor(L64, dtype=torch.float32), as_colmajor(Lb64, dtype=torch.float32))
    torch.cuda.synchronize()
    assert float((got.double() - ref).norm() / ref.norm()) < 1e-4


@pytest.mark.parametrize("n,tol", [(257, 1e-3), (8192, 5e-2)])
def test_sgp_loss_grad_matches_fp64(handle, n, tol):
    g = torch.Generator(device="cuda").manual_seed(5)
    X32 = torch.rand((3, n), generator=g, device="cuda", dtype=torch.float32).t()
    y32 = torch.randn(n, generator=g, device="cuda", dtype=torch.float32)
    X64 = X32.double().t().contiguous().t()
    y64 = y32.double()
    l64, d64, _ = handle.gp_loss_grad(X64, y64, 0.2)
    l32, d32, _ = handle.sgp_loss_grad(X32, y32, 0.2)
    assert abs(l32 - l64) <= tol * abs(l64), (l32, l64)
    assert abs(d32 - d64) <= tol * abs(d64), (d32, d64)
