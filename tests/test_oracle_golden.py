"""The oracle (CPU restatement of Mat-8.3.1) pinned against golden fixtures
produced by the reference itself (tests/golden/make_golden.py): bit-exact
equality (full arrays or SHA-256 of the raw column-major bytes), including the
benchmark sizes n = 8192 (PLU, LLT) and M=N=K=1024 (GEMM)."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from oracle.api import host_fill_normal, host_fill_uniform
from oracle.api import reference, restatement

G = Path(__file__).resolve().parent / "golden"
META = json.loads((G / "golden.json").read_text())["cases"]


def sha(a):
    return hashlib.sha256(np.asfortranarray(a).tobytes(order="F")).hexdigest()


def spd(n, seed):
    """The golden script's S = G G^T / n + I (fused-chain product, then 1/n)."""
    g = host_fill_normal(n, n, seed)
    s = restatement().dgemm(g, np.asfortranarray(g.T)) * (1.0 / n)
    s[np.diag_indices(n)] += 1.0
    return np.asfortranarray(s)


@pytest.fixture(scope="module")
def orc():
    o = restatement()
    o.set_threads(8)
    return o


def test_gemm(orc):
    c = orc.dgemm(host_fill_uniform(61, 90, 2), host_fill_uniform(90, 97, 3))
    assert np.array_equal(c, np.load(G / "gemm_61x97x90.npz")["c"])
    c = orc.dgemm(host_fill_uniform(1024, 1024, 0), host_fill_uniform(1024, 1024, 1))
    assert sha(c) == META["gemm_1024"]["sha256"]


@pytest.mark.parametrize("n", [61, 97])
def test_plu_small(orc, n):
    pos, L, U = orc.plu(host_fill_normal(n, n, 1))
    f = np.load(G / f"plu_{n}.npz")
    assert np.array_equal(pos, f["pos"]) and np.array_equal(L, f["L"]) and np.array_equal(U, f["U"])


@pytest.mark.parametrize("n", [257, 1000, 8192])
def test_plu_digest(orc, n):
    pos, L, U = orc.plu(host_fill_normal(n, n, 1))
    assert np.array_equal(pos, np.load(G / f"plu_{n}_pos.npy"))
    assert sha(L) == META[f"plu_{n}"]["sha256_L"] and sha(U) == META[f"plu_{n}"]["sha256_U"]


@pytest.mark.parametrize("n,k", [(300, 4), (2048, 1), (50, 9), (300, 8), (300, 13), (1000, 150)])
def test_solve_digest(orc, n, k):
    x = orc.solve(host_fill_normal(n, n, 1), host_fill_normal(n, k, 2))
    assert sha(x) == META[f"solve_{n}_{k}"]["sha256"]


def test_lu_without_pivoting(orc):
    def dd(n):
        g = host_fill_normal(n, n, 4)
        g[np.diag_indices(n)] += n
        return np.asfortranarray(g)

    f = np.load(G / "lu_90.npz")
    L, U = orc.lu(dd(90))
    assert np.array_equal(L, f["L"]) and np.array_equal(U, f["U"])
    for n in (300, 1000):
        L, U = orc.lu(dd(n))
        assert sha(L) == META[f"lu_{n}"]["sha256_L"] and sha(U) == META[f"lu_{n}"]["sha256_U"]


def sym(n, seed):
    g = host_fill_normal(n, n, seed)
    return np.asfortranarray(g + g.T)


def test_ldlt(orc):
    f = np.load(G / "ldlt_90.npz")
    L, D = orc.ldlt(sym(90, 3))
    assert np.array_equal(L, f["L"]) and np.array_equal(np.diag(D), f["d"])
    for n in (97, 300, 1000):
        L, D = orc.ldlt(sym(n, 3))
        assert sha(L) == META[f"ldlt_{n}"]["sha256_L"] and sha(np.diag(D)[:, None]) == META[f"ldlt_{n}"]["sha256_d"]


def test_inv(orc):
    assert np.array_equal(orc.inv(host_fill_normal(61, 61, 9)), np.load(G / "inv_61.npz")["X"])
    for n in (97, 300, 1000):
        assert sha(orc.inv(host_fill_normal(n, n, 9))) == META[f"inv_{n}"]["sha256"]


def test_llt(orc):
    assert np.array_equal(orc.llt(spd(97, 1)), np.load(G / "llt_97.npz")["L"])
    for n in (300, 8192):
        assert sha(orc.llt(spd(n, 1))) == META[f"llt_{n}"]["sha256"]


def test_qr(orc):
    q, r = orc.qr(host_fill_normal(60, 40, 7))
    f = np.load(G / "qr_60x40.npz")
    assert np.array_equal(q, f["Q"]) and np.array_equal(r, f["R"])
    for m, n in ((300, 200), (1000, 500)):
        q, r = orc.qr(host_fill_normal(m, n, 7))
        assert sha(q) == META[f"qr_{m}x{n}"]["sha256_Q"] and sha(r) == META[f"qr_{m}x{n}"]["sha256_R"]


def test_det(orc):
    d = orc.det(host_fill_normal(150, 150, 5))
    assert d == META["det_150"]["value"]


@pytest.mark.skipif(reference() is None, reason="reference tree not present (GPU host)")
@pytest.mark.parametrize("m,n", [(7, 7), (91, 91), (130, 61), (500, 500)])
def test_restatement_equals_reference_build(orc, m, n):
    """Where the reference compiles (this container), compare on extra shapes."""
    ref = reference()
    a = host_fill_normal(m, n, 11)
    p1, l1, u1 = orc.plu(a)
    p2, l2, u2 = ref.plu(a)
    assert np.array_equal(p1, p2) and np.array_equal(l1, l2) and np.array_equal(u1, u2)
    q1, r1 = orc.qr(a)
    q2, r2 = ref.qr(a)
    assert np.array_equal(q1, q2) and np.array_equal(r1, r2)
    if m == n:
        s = spd(n, 12)
        assert np.array_equal(orc.llt(s), ref.llt(s))
        assert np.array_equal(orc.inv(a), ref.inv(a))
        for x, y in zip(orc.ldlt(s), ref.ldlt(s)):
            assert np.array_equal(x, y)
        for x, y in zip(orc.lu(a), ref.lu(a)):
            assert np.array_equal(x, y)
        for k in (3, 8, 11):
            if k >= 8 and 60 < n <= 90:
                continue  # the reference's one-block 8-column path overruns its 60-row buffer there
            b = host_fill_normal(n, k, 13)
            assert np.array_equal(orc.solve(a, b), ref.solve(a, b))


# ---------------------------------------------------------------- Mat-8.1 EVD_Q
EVD_EPS = json.loads((G / "golden.json").read_text())["evd81"]["eps"]


def sym(n, seed):
    g = host_fill_normal(n, n, seed)
    return np.asfortranarray(g + g.T)


def test_tridiag81_and_evd_q81(orc):
    """The Mat-8.1 tridiagonalisation and EVD_Q (EVD_QR) bit for bit: n = 37 in
    full, n = 64, 200, 500, 1000 by digest."""
    f = np.load(G / "evd81_37.npz")
    q, d, e = orc.tridiag81(sym(37, 21))
    assert np.array_equal(q, f["Q"]) and np.array_equal(d, f["d"]) and np.array_equal(e, f["e"])
    w, qe = orc.evd_q81(sym(37, 21), EVD_EPS)
    assert np.array_equal(w, f["w"]) and np.array_equal(qe, f["Qe"])
    for n in (64, 200, 500, 1000):
        q, d, e = orc.tridiag81(sym(n, 21))
        c = META[f"tridiag81_{n}"]
        assert (sha(q), sha(d[:, None]), sha(e[:, None])) == (c["sha256_Q"], c["sha256_d"], c["sha256_e"])
        w, qe = orc.evd_q81(sym(n, 21), EVD_EPS)
        assert (sha(w[:, None]), sha(qe)) == (META[f"evd81_{n}"]["sha256_w"], META[f"evd81_{n}"]["sha256_Q"])


def test_evd_q81_properties(orc):
    """Q^T A Q is the tridiagonal; the eigenpairs satisfy A Q = Q diag(w)."""
    a = sym(150, 5)
    q, d, e = orc.tridiag81(a)
    t = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    assert np.abs(q.T @ q - np.eye(150)).max() < 1e-13
    assert np.abs(q.T @ a @ q - t).max() < 1e-12 * np.abs(a).max()
    w, qe = orc.evd_q81(a, 1e-10)
    assert np.abs(a @ qe - qe * w).max() < 1e-9
    assert np.allclose(np.sort(w), np.linalg.eigvalsh(a), atol=1e-10)


def test_evd_q81_budget():
    """With eps = 0 no off-diagonal ever counts as negligible: Mat would loop
    on; the oracle (like the library) stops after 64 n sweeps."""
    with pytest.raises(RuntimeError):
        restatement().evd_q81(sym(12, 3), 0.0)


@pytest.mark.parametrize("n", [2, 3, 8, 9, 33, 130])
def test_evd81_restatement_equals_reference_build(orc, n):
    from oracle.api import reference81

    ref = reference81()
    if ref is None:
        pytest.skip("the Mat-8.1 reference build needs the reference tree and an x86-64 host")
    a = sym(n, 40 + n)
    for x, y in zip(orc.tridiag81(a), ref.tridiag81(a)):
        assert np.array_equal(x, y)
    for x, y in zip(orc.evd_q81(a, 1e-11), ref.evd_q81(a, 1e-11)):
        assert np.array_equal(x, y)


def test_solve_benchmark_configs(orc):
    """The oracle's Solve_direct on the benchmark systems against the
    reference's digests: n = 8192 with 1 RHS, and the mixed solve's n = 16384
    system with 4 RHS (whose input digest is checked too)."""
    from oracle.api import gen_svd_matrix
    x = orc.solve(host_fill_normal(8192, 8192, 1), host_fill_normal(8192, 1, 2))
    assert sha(x) == META["solve_8192_1"]["sha256"]
    a = gen_svd_matrix(16384, 3, 64, 1e-6)
    assert sha(a) == META["solve_svd_16384_4"]["sha256_A"]
    x = orc.solve(a, host_fill_normal(16384, 4, 11))
    assert sha(x) == META["solve_svd_16384_4"]["sha256"]
