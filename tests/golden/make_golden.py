"""Generates the golden fixtures in this directory by running the reference
itself: Mat-8.3.1 compiled from its own headers into oracle/_ref/libmatref.so
(x86-64 AVX-512 build, the configuration of Mat's published numbers), and the
Mat-8.1 snapshot's EVD_Q path into oracle/_ref/libmat81ref.so.

Inputs come from the library's seeded streams as the oracle regenerates
them (oracle.api.host_fill_*, gen_svd_matrix: bit-identical to the library's
host and GPU generators).  Small cases keep full outputs; the benchmark-size
cases keep SHA-256 digests of the raw column-major output bytes (exact,
size-independent) plus a few sketch values.

Run from the repository root:  python tests/golden/make_golden.py
  --large: only (re)computes the benchmark-configuration cases (the solves
  at n = 8192 x 1 and 16384 x 4 on their benchmark inputs, and the
  Householder QR of 16384 x 4096 with its full Q; about five minutes of the
  single-threaded reference) and merges them into golden.json.
"""
from __future__ import annotations

import hashlib
import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle.api import gen_svd_matrix, host_fill_normal, host_fill_uniform, reference, reference81  # noqa: E402

OUT = Path(__file__).resolve().parent
EVD_EPS = 1e-10  # absolute deflation threshold of the EVD_Q cases


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.asfortranarray(a).tobytes(order="F")).hexdigest()


def sketch(a: np.ndarray, seed: int = 99) -> list:
    """4x4 sketch Omega^T a Psi with seeded +-1 Omega, Psi (for tolerance checks)."""
    rng = np.random.default_rng(seed)
    om = rng.choice([-1.0, 1.0], size=(a.shape[0], 4))
    ps = rng.choice([-1.0, 1.0], size=(a.shape[1], 4))
    return (om.T @ a @ ps).tolist()


def spd(ref, n: int, seed: int) -> np.ndarray:
    """S = G G^T / n + I, G iid N(0,1), formed with the reference's own operator*
    (a fused chain per element) and one rounded multiplication by 1/n: the same
    bits on every host and as mg_gen_spd_gram on the GPU."""
    g = host_fill_normal(n, n, seed)
    s = ref.dgemm(g, np.asfortranarray(g.T)) * (1.0 / n)
    s[np.diag_indices(n)] += 1.0
    return np.asfortranarray(s)


def large(ref):
    """The benchmark configurations themselves: FP64 Solve_direct at n = 8192
    with 1 right-hand side (A, b iid N(0,1), seeds 1, 2), at n = 16384 with 4
    (the mixed solve's system: A = Q1 diag(sigma) Q2 from gen_svd_matrix seed
    3, 64 reflectors per side, sigma 1 .. 1e-6; B iid N(0,1) seed 11), and
    QR(A, Q, R, QR_Householder) of a 16384 x 4096 A iid N(0,1) (seed 1)."""
    out = {}
    t = time.time()
    x = ref.solve(host_fill_normal(8192, 8192, 1), host_fill_normal(8192, 1, 2))
    out["solve_8192_1"] = {"sha256": sha(x), "x0": x[:4, 0].tolist(), "seconds": round(time.time() - t, 1)}
    t = time.time()
    a = gen_svd_matrix(16384, 3, 64, 1e-6)
    b = host_fill_normal(16384, 4, 11)
    x = ref.solve(a, b)
    out["solve_svd_16384_4"] = {"sha256": sha(x), "sha256_A": sha(a), "x0": x[:4, 0].tolist(),
                                "seconds": round(time.time() - t, 1)}
    del a, b, x
    t = time.time()
    q, r = ref.qr(host_fill_normal(16384, 4096, 1))
    out["qr_16384x4096"] = {"sha256_Q": sha(q), "sha256_R": sha(r), "sketch_R": sketch(r),
                            "seconds": round(time.time() - t, 1)}
    return out


def main():
    ref = reference()
    if ref is None:
        raise SystemExit("the reference build (oracle/_ref) needs the reference tree and an x86-64 host")
    if "--large" in sys.argv:
        path = OUT / "golden.json"
        meta = json.loads(path.read_text())
        meta["cases"].update(large(ref))
        path.write_text(json.dumps(meta, indent=1))
        print("benchmark-configuration cases merged into golden.json")
        return
    main_all(ref)


def main_all(ref):
    ref = reference()
    if ref is None:
        raise SystemExit("the reference build (oracle/_ref) needs the reference tree and an x86-64 host")
    meta = {"generator": "tests/golden/make_golden.py", "reference": "Mat-8.3.1 (AVX-512 build)", "cases": {}}
    t0 = time.time()

    # GEMM, benchmark configuration M=N=K=1024, A, B uniform [-1,1) seeds 0, 1 (row-major stream)
    a = host_fill_uniform(1024, 1024, 0)
    b = host_fill_uniform(1024, 1024, 1)
    c = ref.dgemm(a, b)
    meta["cases"]["gemm_1024"] = {"sha256": sha(c), "sum": float(c.sum()), "sketch": sketch(c)}
    a = host_fill_uniform(61, 90, 2)
    b = host_fill_uniform(90, 97, 3)
    np.savez_compressed(OUT / "gemm_61x97x90.npz", c=ref.dgemm(a, b))

    # PLU: full factors for small n, digests for larger
    for n in (61, 97):
        pos, L, U = ref.plu(host_fill_normal(n, n, 1))
        np.savez_compressed(OUT / f"plu_{n}.npz", pos=pos, L=L, U=U)
    for n in (257, 1000, 8192):
        pos, L, U = ref.plu(host_fill_normal(n, n, 1))
        np.save(OUT / f"plu_{n}_pos.npy", pos.astype(np.int32))
        meta["cases"][f"plu_{n}"] = {"sha256_L": sha(L), "sha256_U": sha(U), "sketch_L": sketch(L),
                                     "sketch_U": sketch(U)}

    # Solve_direct: narrow path (1 and 4 right-hand sides); wide path with one
    # block (n <= 90), blocked by 60 rows, 8-column groups plus ragged columns,
    # more than one 144-column tile
    for n, k in ((300, 4), (2048, 1), (50, 9), (300, 8), (300, 13), (1000, 150), (8192, 16)):
        x = ref.solve(host_fill_normal(n, n, 1), host_fill_normal(n, k, 2))
        meta["cases"][f"solve_{n}_{k}"] = {"sha256": sha(x), "x0": x[:4, 0].tolist()}

    # LLT: S = G G^T / n + I
    np.savez_compressed(OUT / "llt_97.npz", L=ref.llt(spd(ref, 97, 1)))
    for n in (300, 8192):
        L = ref.llt(spd(ref, n, 1))
        meta["cases"][f"llt_{n}"] = {"sha256": sha(L), "sketch": sketch(L)}

    # QR (Householder): unblocked path in full, blocked path by digest
    q, r = ref.qr(host_fill_normal(60, 40, 7))
    np.savez_compressed(OUT / "qr_60x40.npz", Q=q, R=r)
    for m, n in ((300, 200), (1000, 500)):
        q, r = ref.qr(host_fill_normal(m, n, 7))
        meta["cases"][f"qr_{m}x{n}"] = {"sha256_Q": sha(q), "sha256_R": sha(r), "sketch_R": sketch(r)}

    # Det
    meta["cases"]["det_150"] = {"value": ref.det(host_fill_normal(150, 150, 5))}

    # LU without pivoting: diagonally dominant G + n I, one block in full, blocked by digest
    def dd(n, seed):
        g = host_fill_normal(n, n, seed)
        g[np.diag_indices(n)] += n
        return np.asfortranarray(g)

    L, U = ref.lu(dd(90, 4))
    np.savez_compressed(OUT / "lu_90.npz", L=L, U=U)
    for n in (300, 1000):
        L, U = ref.lu(dd(n, 4))
        meta["cases"][f"lu_{n}"] = {"sha256_L": sha(L), "sha256_U": sha(U)}

    # LDLT: symmetric indefinite G + G^T (no pivoting), one block in full, blocked by digest
    def sym(n, seed):
        g = host_fill_normal(n, n, seed)
        return np.asfortranarray(g + g.T)

    L, D = ref.ldlt(sym(90, 3))
    np.savez_compressed(OUT / "ldlt_90.npz", L=L, d=np.diag(D))
    for n in (97, 300, 1000):
        L, D = ref.ldlt(sym(n, 3))
        meta["cases"][f"ldlt_{n}"] = {"sha256_L": sha(L), "sha256_d": sha(np.diag(D)[:, None])}
    L, D = ref.ldlt(spd(ref, 2048, 1))
    meta["cases"]["ldlt_spd_2048"] = {"sha256_L": sha(L), "sha256_d": sha(np.diag(D)[:, None])}

    # Inv: one block (n <= 90) in full; blocked by 60 by digest
    np.savez_compressed(OUT / "inv_61.npz", X=ref.inv(host_fill_normal(61, 61, 9)))
    for n in (97, 300, 1000, 2048):
        x = ref.inv(host_fill_normal(n, n, 9))
        meta["cases"][f"inv_{n}"] = {"sha256": sha(x), "sketch": sketch(x)}

    # EVD_Q of the Mat-8.1 snapshot (oracle/_ref/libmat81ref.so): symmetric G + G^T;
    # tridiagonalisation (Q, d, e) and the whole EVD_Q with EVD_QR (w, Q) at an
    # absolute deflation threshold; one case in full, larger ones by digest
    ref81 = reference81()
    if ref81 is None:
        raise SystemExit("the Mat-8.1 reference build (oracle/_ref/libmat81ref.so) is missing")
    meta["evd81"] = {"reference": "Mat-8.1 snapshot (AVX-512 build)", "eps": EVD_EPS}
    q, d, e = ref81.tridiag81(sym(37, 21))
    w, qe = ref81.evd_q81(sym(37, 21), EVD_EPS)
    np.savez_compressed(OUT / "evd81_37.npz", Q=q, d=d, e=e, w=w, Qe=qe)
    for n in (64, 200, 500, 1000):
        q, d, e = ref81.tridiag81(sym(n, 21))
        w, qe = ref81.evd_q81(sym(n, 21), EVD_EPS)
        meta["cases"][f"tridiag81_{n}"] = {"sha256_Q": sha(q), "sha256_d": sha(d[:, None]),
                                           "sha256_e": sha(e[:, None])}
        meta["cases"][f"evd81_{n}"] = {"sha256_w": sha(w[:, None]), "sha256_Q": sha(qe)}

    meta["seconds"] = round(time.time() - t0, 1)
    (OUT / "golden.json").write_text(json.dumps(meta, indent=1))
    print(f"golden fixtures written in {meta['seconds']} s")


if __name__ == "__main__":
    main()
