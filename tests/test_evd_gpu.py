"""EVD_Q(A, E, Q, eps, EVD_QR) of the Mat-8.1 snapshot on the GPU: the
Householder tridiagonalisation with its Q and the whole eigendecomposition,
bit for bit against the oracle (itself pinned to the Mat-8.1 build by the
golden fixtures) and the fixtures; properties at larger sizes; the sweep
budget and argument checks."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest
import torch

from mat_gb300 import MatGpuError
from mat_gb300.api import as_colmajor, host_fill_normal
from oracle.api import restatement

pytestmark = pytest.mark.gpu
G = Path(__file__).resolve().parent / "golden"
GOLD = json.loads((G / "golden.json").read_text())
META = GOLD["cases"]
EPS = GOLD["evd81"]["eps"]


def sha(a):
    return hashlib.sha256(np.asfortranarray(a).tobytes(order="F")).hexdigest()


def sym(n, seed):
    g = host_fill_normal(n, n, seed)
    return np.asfortranarray(g + g.T)


def gpu_tridiag(handle, a):
    A = as_colmajor(torch.from_numpy(a))
    Q, d, e = handle.dtridiag81(A)
    torch.cuda.synchronize()
    return Q.cpu().numpy(), d.cpu().numpy(), e.cpu().numpy()


def gpu_evd(handle, a, eps):
    A = as_colmajor(torch.from_numpy(a))
    w, E, Q = handle.devd_q(A, eps)
    torch.cuda.synchronize()
    return w.cpu().numpy(), E.cpu().numpy(), Q.cpu().numpy()


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 8, 9, 17, 33, 64, 100, 257, 1000])
def test_tridiag81_bit_identical(handle, n):
    a = sym(n, 30 + n)
    q, d, e = gpu_tridiag(handle, a)
    q0, d0, e0 = restatement().tridiag81(a)
    assert np.array_equal(d, d0) and np.array_equal(e, e0) and np.array_equal(q, q0)


def test_tridiag81_golden(handle):
    f = np.load(G / "evd81_37.npz")
    q, d, e = gpu_tridiag(handle, sym(37, 21))
    assert np.array_equal(q, f["Q"]) and np.array_equal(d, f["d"]) and np.array_equal(e, f["e"])
    for n in (64, 200, 500, 1000):
        q, d, e = gpu_tridiag(handle, sym(n, 21))
        c = META[f"tridiag81_{n}"]
        assert (sha(q), sha(d[:, None]), sha(e[:, None])) == (c["sha256_Q"], c["sha256_d"], c["sha256_e"])


def test_tridiag81_reads_lower_triangle_only(handle):
    a = sym(130, 7)
    junk = a.copy(order="F")
    junk[np.triu_indices(130, 1)] = np.nan
    q, d, e = gpu_tridiag(handle, junk)
    q0, d0, e0 = restatement().tridiag81(a)
    assert np.array_equal(d, d0) and np.array_equal(e, e0) and np.array_equal(q, q0)


@pytest.mark.parametrize("n", [1, 2, 3, 7, 37, 64, 200, 500, 1000])
def test_evd_q81_bit_identical(handle, n):
    a = sym(n, 21)
    w, E, Q = gpu_evd(handle, a, EPS)
    w0, Q0 = restatement().evd_q81(a, EPS)
    assert np.array_equal(w, w0) and np.array_equal(Q, Q0)
    assert np.array_equal(E, np.diag(w0))
    if f"evd81_{n}" in META:
        assert (sha(w[:, None]), sha(Q)) == (META[f"evd81_{n}"]["sha256_w"], META[f"evd81_{n}"]["sha256_Q"])
    if n == 37:
        f = np.load(G / "evd81_37.npz")
        assert np.array_equal(w, f["w"]) and np.array_equal(Q, f["Qe"])


def test_evd_q81_bit_identical_1000(handle):
    """Several rotation chunks' worth of sweeps on the GPU (n = 1000)."""
    a = sym(1000, 8)
    w, _, Q = gpu_evd(handle, a, 1e-9)
    w0, Q0 = restatement().evd_q81(a, 1e-9)
    assert np.array_equal(w, w0) and np.array_equal(Q, Q0)


@pytest.mark.parametrize("n", [2048])
def test_evd_q81_properties(handle, n):
    """At a larger size: Q orthogonal, A Q = Q diag(w), eigenvalues of A."""
    a = sym(n, 3)
    eps = 1e-11  # absolute deflation threshold: the eigenpair residuals are of this order
    w, _, Q = gpu_evd(handle, a, eps)
    At = torch.from_numpy(a).cuda()
    Qt = torch.from_numpy(Q).cuda()
    wt = torch.from_numpy(w).cuda()
    assert (Qt.T @ Qt - torch.eye(n, dtype=torch.float64, device="cuda")).abs().max().item() < 1e-12
    assert (At @ Qt - Qt * wt).abs().max().item() < 100 * eps
    ref = torch.linalg.eigvalsh(At).cpu().numpy()
    assert np.abs(np.sort(w) - ref).max() < 100 * eps


def test_evd_q81_sweep_budget(handle):
    """eps = 0: nothing deflates; Mat loops on, the library stops after 64 n sweeps."""
    with pytest.raises(MatGpuError):
        gpu_evd(handle, sym(12, 3), 0.0)
    # the handle stays usable
    a = sym(9, 1)
    w, _, Q = gpu_evd(handle, a, EPS)
    w0, Q0 = restatement().evd_q81(a, EPS)
    assert np.array_equal(w, w0) and np.array_equal(Q, Q0)


def test_evd_q81_bad_arguments(handle):
    A = as_colmajor(torch.from_numpy(sym(8, 1)))
    with pytest.raises(MatGpuError):
        handle.devd_q(A, -1.0)


@pytest.mark.parametrize("cap", ["0", "100"])
def test_tridiag81_global_memory_path(handle, monkeypatch, cap):
    """Above the on-chip capacity (n > 4097) the update reads v, w and the first
    column from global memory; the test hook lowers the threshold so both paths
    (all steps, or the first ones) run at a small size, bit for bit."""
    monkeypatch.setenv("MG_TRIDIAG_STAGE_CAP", cap)
    a = sym(300, 17)
    q, d, e = gpu_tridiag(handle, a)
    q0, d0, e0 = restatement().tridiag81(a)
    assert np.array_equal(d, d0) and np.array_equal(e, e0) and np.array_equal(q, q0)


def test_formq81_global_memory_kernel(handle, monkeypatch):
    """Q from the reflectors with the global-memory kernel (used above n = 4096),
    forced at a small size by the test hook, bit for bit."""
    monkeypatch.setenv("MG_FORMQ_NMAX", "0")
    a = sym(300, 19)
    q, d, e = gpu_tridiag(handle, a)
    q0, d0, e0 = restatement().tridiag81(a)
    assert np.array_equal(d, d0) and np.array_equal(e, e0) and np.array_equal(q, q0)


def test_tridiag81_large_properties(handle):
    """n = 4200: the first steps exceed the on-chip capacity (global-memory
    update) and Q is formed by the global-memory kernel; Q orthogonal and
    Q^T A Q tridiagonal with the returned d, e."""
    n = 4200
    a = sym(n, 23)
    At = torch.from_numpy(a).cuda()
    A = At.t().contiguous().t().clone()
    Q, d, e = handle.dtridiag81(A)
    torch.cuda.synchronize()
    T = torch.diag(d) + torch.diag(e, 1) + torch.diag(e, -1)
    nrm = At.abs().max().item()
    assert (Q.T @ Q - torch.eye(n, dtype=torch.float64, device="cuda")).abs().max().item() < 1e-12
    assert (Q.T @ At @ Q - T).abs().max().item() < 1e-11 * nrm * 10


def test_evd_q81_in_place(handle):
    """A == E (Mat allows EVD_Q(A, A, Q, ...)): the same result, E overwritten."""
    a = sym(97, 29)
    A = as_colmajor(torch.from_numpy(a))
    w, E, Q = handle.devd_q(A, EPS, E=A)
    torch.cuda.synchronize()
    w0, Q0 = restatement().evd_q81(a, EPS)
    assert E.data_ptr() == A.data_ptr()
    assert np.array_equal(w.cpu().numpy(), w0) and np.array_equal(Q.cpu().numpy(), Q0)
    assert np.array_equal(A.cpu().numpy(), np.diag(w0))
