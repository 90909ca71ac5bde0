"""The host half of EVD_Q (the QR sweeps' scalar recurrence, run on the host
by mg_devd_q while the GPU applies the rotations) against the oracle, on the
CPU: eigenvalues bit for bit from the oracle's tridiagonal, the rotation
count, the sweep budget and argument checks."""
import numpy as np
import pytest

from mat_gb300 import MatGpuError
from mat_gb300.api import host_fill_normal, host_steqr81
from oracle.api import restatement


def sym(n, seed):
    g = host_fill_normal(n, n, seed)
    return np.asfortranarray(g + g.T)


@pytest.mark.parametrize("n", [1, 2, 3, 5, 16, 37, 130, 400])
def test_steqr81_host_matches_oracle(n):
    a = sym(n, 50 + n)
    _, d, e = restatement().tridiag81(a)
    w, nrot = host_steqr81(d, e, 1e-10)
    w0, _ = restatement().evd_q81(a, 1e-10)
    assert np.array_equal(w, w0)
    assert (nrot == 0) == (n == 1)


def test_steqr81_host_budget_and_arguments():
    _, d, e = restatement().tridiag81(sym(12, 3))
    with pytest.raises(MatGpuError):
        host_steqr81(d, e, 0.0)  # nothing deflates at eps = 0
    with pytest.raises(MatGpuError):
        host_steqr81(d, e, -1.0)
