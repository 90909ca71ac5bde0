"""FP64 GEMM on the GPU against an FP64 host product (numpy) of the same
seeded inputs; tolerance 1e-13 normwise relative (Mat operator* parity bar)."""
import numpy as np
import pytest
import torch

from mat_gb300.api import as_colmajor, colmajor, host_fill_normal, host_fill_uniform

pytestmark = pytest.mark.gpu
TOL = 1e-13


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_device_generators_match_host(handle):
    for (r, c) in [(1, 1), (33, 17), (256, 129)]:
        for rm in (True, False):
            d = colmajor(r, c)
            handle.fill_uniform(d, seed=7, rowmajor_stream=rm)
            assert np.array_equal(d.cpu().numpy(), host_fill_uniform(r, c, 7, rowmajor_stream=rm))
            handle.fill_normal(d, seed=9, rowmajor_stream=rm)
            assert np.array_equal(d.cpu().numpy(), host_fill_normal(r, c, 9, rowmajor_stream=rm))


@pytest.mark.parametrize("m,n,k", [(1, 1, 1), (7, 5, 3), (61, 97, 90), (128, 128, 16), (129, 257, 33),
                                   (300, 200, 500), (1024, 1024, 1024)])
@pytest.mark.parametrize("ta,tb", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_dgemm_matches_fp64_product(handle, m, n, k, ta, tb):
    a = host_fill_uniform(k if ta else m, m if ta else k, seed=0)
    b = host_fill_uniform(n if tb else k, k if tb else n, seed=1)
    c0 = host_fill_uniform(m, n, seed=2)
    A, B, Cd = as_colmajor(torch.from_numpy(a)), as_colmajor(torch.from_numpy(b)), as_colmajor(torch.from_numpy(c0))
    opa = a.T if ta else a
    opb = b.T if tb else b
    # beta = 0 (Mat operator*)
    out = handle.dgemm(A, B, transA=bool(ta), transB=bool(tb))
    torch.cuda.synchronize()
    assert rel(out.cpu().numpy(), opa @ opb) < TOL
    # subtracting update (alpha=-1, beta=1): __mulAB_packed_n
    handle.dgemm(A, B, Cd, alpha=-1.0, beta=1.0, transA=bool(ta), transB=bool(tb))
    torch.cuda.synchronize()
    assert rel(Cd.cpu().numpy(), c0 - opa @ opb) < TOL


def test_dgemm_odd_ld_submatrix(handle):
    # sub-matrix views with odd leading dimension and odd offsets
    big = as_colmajor(torch.from_numpy(host_fill_uniform(301, 300, seed=3)))
    A = big[3:200, 5:120]
    B = big[1:116, 7:99]
    out = handle.dgemm(A, B)
    torch.cuda.synchronize()
    ref = A.cpu().numpy() @ B.cpu().numpy()
    assert rel(out.cpu().numpy(), ref) < TOL


def test_dgemm_beta0_ignores_nan(handle):
    A = as_colmajor(torch.from_numpy(host_fill_uniform(64, 64, seed=4)))
    Cd = colmajor(64, 64)
    Cd.fill_(float("nan"))
    handle.dgemm(A, A, Cd, alpha=1.0, beta=0.0)
    torch.cuda.synchronize()
    assert torch.isfinite(Cd).all()
