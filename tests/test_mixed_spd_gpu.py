"""Mixed-precision SPD solve (mg_dsposv_ir): fp32 Cholesky with split-BF16
tensor-core trailing updates, the factor rewritten as the packed LU of the
same matrix, then the FP64 refinement of the mixed LU solve.  Checked on
Gram matrices G G^T / n + I and on the Gaussian-process kernel of the
differentiated-Cholesky configuration (RBF, lengthscale 0.2, unit
variance, 1e-2 jitter, points in [0,1]^3): normwise backward error <= 1e-14
recomputed in FP64, agreement with the FP64 GPU Cholesky solve; and the
breakdown path (an indefinite matrix: MG_NOT_SPD without the fallback, the
FP64 solve with it)."""
import ctypes as C

import numpy as np
import pytest
import torch

from mat_gb300._lib import IrOpts, IrReport
from mat_gb300.api import colmajor

pytestmark = pytest.mark.gpu


def backward_error(a, x, b):
    r = b - a @ x
    return (np.abs(r).max(0) / (np.abs(a).sum(1).max() * np.abs(x).max(0) + np.abs(b).max(0))).max()


def fp64_chol_solve(handle, S, B):
    L = S.clone()
    assert handle.dpotrf(L) == 0
    return handle.dpotrs(L, B.clone())


# 50: one diagonal block only; 65: a one-row block column; 128: two blocks,
# no far update; 129: a far update of one row; then ragged last blocks
@pytest.mark.parametrize("n,nrhs", [(50, 2), (65, 1), (128, 1), (129, 3), (300, 1), (1000, 4), (2500, 3), (4096, 4)])
def test_mixed_spd_gram(handle, n, nrhs):
    S = colmajor(n, n)
    handle.gen_spd_gram(S, 1)
    B = colmajor(n, nrhs)
    handle.fill_normal(B, 2)
    X, rep = handle.dsposv_ir(S, B)
    torch.cuda.synchronize()
    assert rep["status"] == 0 and rep["path"] == 0, rep
    s, b, x = S.cpu().numpy(), B.cpu().numpy(), X.cpu().numpy()
    assert backward_error(s, x, b) <= 1e-14
    xd = fp64_chol_solve(handle, S, B).cpu().numpy()
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-12


@pytest.mark.parametrize("n", [2048, 8192])
def test_mixed_spd_gp_kernel(handle, n):
    g = torch.Generator(device="cuda").manual_seed(5)
    Xp = torch.rand((3, n), generator=g, device="cuda", dtype=torch.float64).t()
    K = handle.gen_rbf_kernel(Xp, 0.2, 1.0, 1e-2)
    y = colmajor(n, 1)
    handle.fill_normal(y, 6)
    X, rep = handle.dsposv_ir(K, y)
    torch.cuda.synchronize()
    assert rep["status"] == 0 and rep["path"] == 0 and rep["iterations"] <= 6, rep
    k, b, x = K.cpu().numpy(), y.cpu().numpy(), X.cpu().numpy()
    assert backward_error(k, x, b) <= 1e-14


def test_mixed_spd_breakdown(handle):
    n = 500
    A = colmajor(n, n)
    handle.fill_normal(A, 3)
    S = (A + A.t()).t().contiguous().t()  # symmetric indefinite
    B = colmajor(n, 2)
    handle.fill_normal(B, 4)
    X = colmajor(n, 2)
    o = IrOpts(1e-14, 30, 3, 0, 1, 0, 0)  # no fallback
    r = IrReport()
    st = handle.lib.mg_dsposv_ir(handle.h, n, 2, C.c_void_p(S.data_ptr()), n, C.c_void_p(B.data_ptr()), n,
                                 C.c_void_p(X.data_ptr()), n, C.byref(o), C.byref(r))
    assert st == 5 and r.info >= 1  # MG_NOT_SPD, the column where the fp32 Cholesky broke down
    X2, rep = handle.dsposv_ir(S, B)  # with the FP64 fallback
    torch.cuda.synchronize()
    assert rep["status"] == 7 and rep["path"] == 2, rep
    assert backward_error(S.cpu().numpy(), X2.cpu().numpy(), B.cpu().numpy()) <= 1e-14
