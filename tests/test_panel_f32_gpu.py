"""FP32 LU of the mixed solve: the panel (mg_sgetf2) against a restatement of
the fp32 partial-pivoting LU with exactly rounded fused updates, on the
cluster path (m <= 16384; clusters of 1, 2, 4, 8 and 16 CTAs, 1..4 rows
per thread, ragged sub-panels, clusters with idle CTAs) and the
cooperative-grid path (m > 16384); exact zero columns and tied candidates;
and the blocked mg_sgetrf by its defining
properties (|L| <= 1, P A = L U to fp32 accuracy).
"""
import numpy as np
import pytest
import torch

from mat_gb300.api import as_colmajor

pytestmark = pytest.mark.gpu

F32 = torch.float32


def sgetf2_restated(a32: np.ndarray):
    """fp32 getf2: first index of max |a|, reciprocal (correctly rounded),
    fp32 multiply, then a := fma(l, -u, a) rounded once to fp32 (emulated in
    float64: the product of two fp32 values is exact there)."""
    a = a32.astype(np.float64)
    m, n = a.shape
    perm = np.arange(m)
    info = 0
    for c in range(min(m, n)):
        col = np.abs(a[c:, c])
        k = int(np.argmax(col)) + c
        if not col[k - c] > 0:
            info = info or c + 1
            continue
        if k != c:
            a[[c, k], :] = a[[k, c], :]
            perm[[c, k]] = perm[[k, c]]
        inv = np.float32(1.0) / np.float32(a[c, c])
        l = (a[c + 1:, c].astype(np.float32) * inv).astype(np.float64)
        a[c + 1:, c] = l
        a[c + 1:, c + 1:] = (a[c + 1:, c + 1:] - np.outer(l, a[c, c + 1:])).astype(np.float32).astype(np.float64)
    return a.astype(np.float32), perm, info


def run_panel(handle, a: np.ndarray):
    A = as_colmajor(torch.from_numpy(a), dtype=F32)
    pos, info = handle.sgetf2(A)
    torch.cuda.synchronize()
    return A.cpu().numpy(), pos.cpu().numpy(), info


@pytest.mark.parametrize("m,n", [(300, 128), (4096, 128), (5000, 128), (9000, 101), (16384, 128), (3000, 77),
                                 (20000, 100), (128, 128), (700, 40), (1000, 1), (777, 17), (1025, 128),
                                 (1800, 128), (2048, 64), (8192, 128), (8193, 96)])
def test_sgetf2_matches_restatement(handle, m, n):
    rng = np.random.default_rng(m * 131 + n)
    a = rng.standard_normal((m, n)).astype(np.float32)
    got, pos, info = run_panel(handle, a)
    ref, perm, rinfo = sgetf2_restated(a)
    assert info == rinfo == 0
    np.testing.assert_array_equal(pos, perm)
    # bitwise up to the rare double rounding of the float64 emulation
    diff = np.abs(got.astype(np.float64) - ref.astype(np.float64))
    assert diff.max() <= 1e-5 * np.abs(ref).max(), diff.max()
    assert (diff != 0).mean() < 1e-4


def test_sgetf2_zero_column_and_ties(handle):
    m, n = 6000, 96
    rng = np.random.default_rng(5)
    a = rng.standard_normal((m, n)).astype(np.float32)
    a[:, 40] = 0.0                 # exactly zero column -> info 41, no interchange
    a[4500, 0] = 50.0              # tied largest |a| in column 0: first row wins
    a[3000, 0] = -50.0
    a[[1200, 5900], 7] = [40.0, 40.0]
    got, pos, info = run_panel(handle, a)
    ref, perm, rinfo = sgetf2_restated(a)
    assert rinfo == 41 and info == 41
    assert pos[0] == 3000
    np.testing.assert_array_equal(pos, perm)
    diff = np.abs(got.astype(np.float64) - ref.astype(np.float64))
    assert diff.max() <= 1e-5 * np.abs(ref).max()


@pytest.mark.parametrize("n", [1000, 4100])
def test_sgetrf_properties(handle, n):
    g = torch.Generator(device="cuda").manual_seed(n)
    A0 = torch.randn(n, n, device="cuda", generator=g, dtype=torch.float64)
    A = as_colmajor(A0, dtype=F32)
    pos, info = handle.sgetrf(A)
    torch.cuda.synchronize()
    assert info == 0
    p = pos.long()
    assert torch.equal(torch.sort(p).values, torch.arange(n, device="cuda"))
    LU = A.double()
    L = torch.tril(LU, -1) + torch.eye(n, device="cuda", dtype=torch.float64)
    U = torch.triu(LU)
    assert L.abs().max().item() <= 1.0 + 1e-6
    PA = A0.to(F32).double()[p]
    rel = (PA - L @ U).abs().max().item() / A0.abs().max().item()
    assert rel < 2e-4 * (n / 1000) ** 0.5, rel
