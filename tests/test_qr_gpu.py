"""Mat QR(A, Q, R, QR_Householder) on the GPU against the oracle, bit for bit
on both of Mat's paths: the blocked one (min(m, n) > 96) and the unblocked
variant Mat uses for smaller min(m, n), which leaves rounding-level values
below R's diagonal (the GPU reproduces them); plus A = QR and Q^T Q = I."""
import numpy as np
import pytest
import torch

from mat_gb300.api import as_colmajor, host_fill_normal
from oracle.api import restatement

pytestmark = pytest.mark.gpu
TOL = 1e-13


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("m,n", [(1, 1), (5, 3), (3, 5), (40, 30), (96, 96), (97, 40), (500, 96), (2000, 64),
                                 (200, 96), (130, 97), (300, 200), (250, 250), (400, 150), (150, 300), (1000, 500)])
def test_qr_matches_oracle(handle, m, n):
    a = host_fill_normal(m, n, seed=7)
    Q, R = handle.dqr(as_colmajor(torch.from_numpy(a)))
    torch.cuda.synchronize()
    q, r = Q.cpu().numpy(), R.cpu().numpy()
    oq, orr = restatement().qr(a)
    assert np.array_equal(r, orr) and np.array_equal(q, oq)
    if min(m, n) > 96:
        assert np.array_equal(np.tril(r, -1), np.zeros_like(r))
    assert rel(q @ r, a) < 1e-14 * max(1.0, m / 100)
    assert np.linalg.norm(q.T @ q - np.eye(m)) < 1e-13 * max(1.0, m / 100)


def test_qr_zero_column(handle):
    a = host_fill_normal(200, 120, seed=8)
    a[:, 50] = 0.0
    Q, R = handle.dqr(as_colmajor(torch.from_numpy(a)))
    torch.cuda.synchronize()
    q, r = Q.cpu().numpy(), R.cpu().numpy()
    assert rel(q @ r, a) < 1e-14
