"""Mixed-precision Householder QR (mg_sgeqrf: fp32 panels with FP64 norm /
beta / tau, split-BF16 tensor-core trailing updates) and the QR-based mixed
solve with FP64 refinement (mg_dsqrsv_ir).

The factorization is checked by its defining properties, in FP64 on the GPU:
A = Q R with Q = H_0 H_1 ... H_{n-1} rebuilt from the stored reflectors and
tau (H = I - tau v v^T, v_c = 1), R upper triangular, to fp32-level accuracy;
|R(c,c)| against the FP64 GPU QR of the same matrix; T of the first panel
such that I - V T V^T = H_0 ... H_127.  The solve reaches normwise backward
error <= 1e-14 (recomputed in FP64) at condition 1e6 and agrees with the
FP64 GPU solve."""
import numpy as np
import pytest
import torch

from mat_gb300.api import colmajor

pytestmark = pytest.mark.gpu


def rebuild(Af, tau):
    """Q R from the packed fp32 factors, in FP64: apply H_{n-1}, ..., H_0 to [R; 0]."""
    m, n = Af.shape
    A = Af.double()
    R = torch.triu(A)[:n, :] if m >= n else torch.triu(A)
    X = torch.zeros((m, n), dtype=torch.float64, device=A.device)
    X[:n, :] = R
    V = torch.tril(A, -1)
    V[range(n), range(n)] = 1.0
    for c in range(n - 1, -1, -1):
        v = V[c:, c]
        X[c:, :] -= tau[c] * torch.outer(v, v @ X[c:, :])
    return X, R, V


@pytest.mark.parametrize("m,n", [(300, 200), (1000, 1000), (4096, 1024), (3000, 257), (9000, 300)])
def test_sgeqrf_reconstructs_A(handle, m, n):
    A = colmajor(m, n)
    handle.fill_normal(A, 7)
    Af = A.float().t().contiguous().t()
    tau, T = handle.sgeqrf(Af)
    torch.cuda.synchronize()
    QR, R, V = rebuild(Af, tau)
    rel = float((A - QR).norm() / A.norm())
    assert rel < 4e-8 * np.sqrt(m * n) ** 0.5 * 10, rel  # fp32 rounding, growing mildly with size
    assert bool((tau >= 0).all()) and bool((tau <= 2).all())
    # |diag R| against the FP64 QR of the same matrix (signs follow the same convention)
    Ad = A.clone()
    taud = torch.empty(n, dtype=torch.float64, device="cuda")
    Td = torch.empty(((n + 47) // 48) * 48 * 48, dtype=torch.float64, device="cuda")
    import ctypes as C
    handle.check(handle.lib.mg_dgeqrf(handle.h, m, n, C.c_void_p(Ad.data_ptr()), m, C.c_void_p(taud.data_ptr()),
                                      C.c_void_p(Td.data_ptr())), "mg_dgeqrf")
    d32, d64 = torch.diagonal(R).abs(), torch.diagonal(Ad).abs()
    assert float(((d32 - d64).abs() / d64).max()) < 1e-3
    # T of the first panel: I - V T V^T equals H_0 ... H_{w-1}
    w = min(128, n)
    Vw = V[:, :w]
    Tw = T[: 128 * 128].view(128, 128).t()[:w, :w].double()  # block stored column-major, ld 128
    e = torch.eye(m, w, dtype=torch.float64, device="cuda")
    lhs = e - Vw @ (Tw @ (Vw.t() @ e))
    rhs = e.clone()
    for c in range(w - 1, -1, -1):
        v = Vw[c:, c]
        rhs[c:, :] -= tau[c] * torch.outer(v, v @ rhs[c:, :])
    assert float((lhs - rhs).abs().max()) < 1e-4


def backward_error(a, x, b):
    r = b - a @ x
    return (np.abs(r).max(0) / (np.abs(a).sum(1).max() * np.abs(x).max(0) + np.abs(b).max(0))).max()


@pytest.mark.parametrize("n,nrhs", [(300, 1), (1024, 4), (2500, 3), (7000, 2)])
def test_mixed_qr_solve(handle, n, nrhs):
    A = colmajor(n, n)
    handle.gen_svd_matrix(A, 3, nrefl=64, sigma_min=1e-6)
    B = colmajor(n, nrhs)
    handle.fill_normal(B, 11)
    X, rep = handle.dsqrsv_ir(A, B)
    torch.cuda.synchronize()
    assert rep["status"] == 0 and rep["path"] == 0, rep
    a, b, x = A.cpu().numpy(), B.cpu().numpy(), X.cpu().numpy()
    assert backward_error(a, x, b) <= 1e-14
    Xd, info = handle.dgesv(A, B)
    xd = Xd.cpu().numpy()
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-8
