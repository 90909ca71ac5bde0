"""ctypes wrappers of the oracle libraries (test infrastructure only).

`Oracle(lib)` wraps either the restatement (liboracle.so, prefix orc_) or the
reference build (_ref/libmatref.so, prefix ref_) behind one numpy API; both
take and return column-major float64 arrays."""
from __future__ import annotations

import ctypes as C
from functools import lru_cache

import numpy as np

from . import build as _build

_P = C.c_void_p


def _f(a):
    a = np.asfortranarray(a, dtype=np.float64)
    return a


def _p(a):
    return a.ctypes.data_as(_P)


class Oracle:
    def __init__(self, path, prefix):
        self.lib = C.CDLL(str(path))
        self.prefix = prefix
        self.is_ref = prefix.startswith("ref")
        if not self.is_ref:
            self.lib.orc_det.restype = C.c_double
            for n in ("orc_dgetrf", "orc_plu", "orc_solve", "orc_llt", "orc_inv", "orc_ldlt", "orc_lu",
                      "orc_evd_q81"):
                getattr(self.lib, n).restype = C.c_int
            self.lib.orc_host_fill_uniform.argtypes = [_P, C.c_int, C.c_int, C.c_int, C.c_uint64, C.c_double,
                                                       C.c_double, C.c_int]
            self.lib.orc_host_fill_uniform.restype = None
            self.lib.orc_host_fill_normal.argtypes = [_P, C.c_int, C.c_int, C.c_int, C.c_uint64, C.c_int]
            self.lib.orc_host_fill_normal.restype = None
            self.lib.orc_gen_svd_matrix.argtypes = [C.c_int, _P, C.c_int, C.c_uint64, C.c_int, C.c_double]
            self.lib.orc_gen_svd_matrix.restype = C.c_int
        elif prefix == "ref_":
            self.lib.ref_det.restype = C.c_double

    def _fn(self, name):
        return getattr(self.lib, self.prefix + name)

    def set_threads(self, n: int):
        if not self.is_ref:
            self.lib.orc_set_threads(int(n))

    def dgemm(self, A, B):
        A, B = _f(A), _f(B)
        m, k = A.shape
        n = B.shape[1]
        Cm = np.zeros((m, n), order="F")
        if self.is_ref:
            self.lib.ref_dgemm(m, n, k, _p(A), _p(B), _p(Cm))
        else:
            self.lib.orc_dgemm(m, n, k, _p(A), max(m, 1), _p(B), max(k, 1), _p(Cm), max(m, 1))
        return Cm

    def plu(self, A):
        """Mat PLU(A, pos, L, U): returns (pos, L, U) with A[pos] == L @ U."""
        A = _f(A)
        m, n = A.shape
        pos = np.zeros(m, dtype=np.int32)
        L = np.zeros((m, m), order="F")
        U = np.zeros((m, n), order="F")
        self._fn("plu")(m, n, _p(A), _p(pos), _p(L), _p(U))
        return pos, L, U

    def solve(self, A, B):
        A, B = _f(A), _f(B)
        n, nrhs = B.shape
        X = np.zeros((n, nrhs), order="F")
        self._fn("solve")(n, nrhs, _p(A), _p(B), _p(X))
        return X

    def inv(self, A):
        """Mat Inv(A) (square)."""
        A = _f(A)
        n = A.shape[0]
        X = np.zeros((n, n), order="F")
        self._fn("inv")(n, _p(A), _p(X))
        return X

    def lu(self, A):
        """Mat LU(A, L, U) without pivoting (square): returns (L, U)."""
        A = _f(A)
        n = A.shape[0]
        L = np.zeros((n, n), order="F")
        U = np.zeros((n, n), order="F")
        self._fn("lu")(n, _p(A), _p(L), _p(U))
        return L, U

    def ldlt(self, A):
        """Mat LDLT(A, L, D): returns (L, D) from A's lower triangle."""
        A = _f(A)
        n = A.shape[0]
        L = np.zeros((n, n), order="F")
        D = np.zeros((n, n), order="F")
        self._fn("ldlt")(n, _p(A), _p(L), _p(D))
        return L, D

    def llt(self, A):
        A = _f(A)
        n = A.shape[0]
        L = np.zeros((n, n), order="F")
        self._fn("llt")(n, _p(A), _p(L))
        return L

    def qr(self, A):
        A = _f(A)
        m, n = A.shape
        Q = np.zeros((m, m), order="F")
        R = np.zeros((m, n), order="F")
        self._fn("qr")(m, n, _p(A), _p(Q), _p(R))
        return Q, R

    def tridiag81(self, A):
        """Mat-8.1 EVD_Q tridiagonalisation: returns (Q, d, e), Q^T A Q = tridiag(e, d, e)."""
        A = _f(A)
        n = A.shape[0]
        Q = np.zeros((n, n), order="F")
        d = np.zeros(n)
        e = np.zeros(max(n - 1, 1))
        if self.is_ref:
            self._fn("tridiag")(n, _p(A), _p(Q), _p(d), _p(e))
        else:
            self.lib.orc_tridiag81(n, _p(A), n, _p(Q), n, _p(d), _p(e))
        return Q, d, e[: n - 1]

    def evd_q81(self, A, eps):
        """Mat-8.1 EVD_Q(A, E, Q, eps, EVD_QR): returns (w, Q), A Q = Q diag(w)."""
        A = _f(A)
        n = A.shape[0]
        Q = np.zeros((n, n), order="F")
        if self.is_ref:
            E = np.zeros((n, n), order="F")
            self._fn("evd_q")(n, _p(A), C.c_double(eps), _p(E), _p(Q))
            return np.diag(E).copy(), Q
        w = np.zeros(n)
        if self.lib.orc_evd_q81(n, _p(A), C.c_double(eps), _p(w), _p(Q)) != 0:
            raise RuntimeError("EVD_Q: QR sweeps did not converge")
        return w, Q

    def det(self, A):
        A = _f(A)
        return float(self._fn("det")(A.shape[0], _p(A)))


@lru_cache(maxsize=None)
def restatement() -> Oracle:
    return Oracle(_build.build_oracle(), "orc_")


@lru_cache(maxsize=None)
def reference() -> Oracle | None:
    lib = _build.build_ref()
    return Oracle(lib, "ref_") if lib else None


@lru_cache(maxsize=None)
def reference81() -> Oracle | None:
    """The Mat-8.1 snapshot's EVD_Q path (entry points prefixed ref81_)."""
    lib = _build.build_ref81()
    return Oracle(lib, "ref81_") if lib else None


def dgemm(A, B):
    return restatement().dgemm(A, B)


# The library's seeded inputs regenerated by the oracle (same streams, same
# bits as mg_host_fill_* and the GPU generators).

def host_fill_uniform(rows: int, cols: int, seed: int, lo=-1.0, hi=1.0, rowmajor_stream=True) -> np.ndarray:
    a = np.empty((rows, cols), order="F")
    if rows and cols:
        restatement().lib.orc_host_fill_uniform(_p(a), rows, cols, max(rows, 1), seed, lo, hi,
                                                int(rowmajor_stream))
    return a


def host_fill_normal(rows: int, cols: int, seed: int, rowmajor_stream=True) -> np.ndarray:
    a = np.empty((rows, cols), order="F")
    if rows and cols:
        restatement().lib.orc_host_fill_normal(_p(a), rows, cols, max(rows, 1), seed, int(rowmajor_stream))
    return a


def gen_svd_matrix(n: int, seed: int, nrefl: int = 64, sigma_min: float = 1e-6) -> np.ndarray:
    """A = Q1 diag(sigma) Q2 as the library's mg_gen_svd_matrix makes it (bit for bit)."""
    a = np.empty((n, n), order="F")
    if restatement().lib.orc_gen_svd_matrix(n, _p(a), max(n, 1), seed, nrefl, sigma_min) != 0:
        raise ValueError("gen_svd_matrix: invalid arguments")
    return a
