"""Split-BF16 tcgen05 GEMM against an fp64 product of the same fp32 inputs.
Tolerances (normwise relative), scaled by sqrt(k/64) for the fp32
accumulation over k: 3 terms ~ fp32 (2e-6), 2 terms ~ 16 bits (1e-4),
1 term = bf16 (1e-2)."""
import numpy as np
import pytest
import torch

from mat_gb300.api import colmajor

pytestmark = pytest.mark.gpu
TOL = {3: 2e-6, 2: 1e-4, 1: 1e-2}


def make(m, n, seed, scale_exp=0):
    g = torch.Generator().manual_seed(seed)
    u = torch.rand(m, n, generator=g, dtype=torch.float64) * 2 - 1
    if scale_exp:
        e = torch.randint(-scale_exp, scale_exp + 1, (m, n), generator=g).to(torch.float64)
        u = u * torch.pow(2.0, e)
    return u.float()


def run(handle, a, b, nterms, c0=None, alpha=1.0, beta=0.0, ordered=False):
    A = a.cuda().t().contiguous().t()
    B = b.cuda().t().contiguous().t()
    Cd = None if c0 is None else c0.cuda().t().contiguous().t()
    out = handle.sgemm_bf16x(A, B, Cd, alpha=alpha, beta=beta, nterms=nterms, ordered=ordered)
    torch.cuda.synchronize()
    return out.cpu().double()


@pytest.mark.parametrize("m,n,k", [(128, 256, 32), (1, 1, 1), (200, 300, 70), (129, 257, 33), (512, 768, 1024),
                                   (1000, 130, 96)])
@pytest.mark.parametrize("nterms", [3, 2, 1])
@pytest.mark.parametrize("ordered", [False, True])
def test_split_gemm_accuracy(handle, m, n, k, nterms, ordered):
    a, b = make(m, k, 1), make(k, n, 2)
    ref = a.double() @ b.double()
    out = run(handle, a, b, nterms, ordered=ordered)
    err = (out - ref).norm() / ref.norm()
    assert err < TOL[nterms] * max(1.0, (k / 64) ** 0.5), float(err)


def test_split_gemm_ordered_is_more_accurate(handle):
    # the lower-order products accumulated before the leading one
    a, b = make(512, 4096, 8, 8), make(4096, 384, 9, 8)
    ref = a.double() @ b.double()
    e1 = float((run(handle, a, b, 3) - ref).norm() / ref.norm())
    e2 = float((run(handle, a, b, 3, ordered=True) - ref).norm() / ref.norm())
    assert e2 < 0.6 * e1, (e2, e1)


def test_split_gemm_wide_exponents(handle):
    # entries u * 2^e, e uniform in [-8, 8] (the M=N=K=16384 configuration's distribution)
    a, b = make(384, 1024, 3, 8), make(1024, 512, 4, 8)
    ref = a.double() @ b.double()
    out = run(handle, a, b, 3)
    assert (out - ref).norm() / ref.norm() < 2e-6 * 4


def test_split_gemm_subtracting_update(handle):
    # the LU trailing update form: C := C - A B
    a, b, c = make(300, 128, 5), make(128, 520, 6), make(300, 520, 7)
    ref = c.double() - a.double() @ b.double()
    for ordered in (False, True):
        out = run(handle, a, b, 3, c0=c, alpha=-1.0, beta=1.0, ordered=ordered)
        assert (out - ref).norm() / ref.norm() < 2e-6
