"""Python mirror of Mat's API for the GPU hot path, over the C ABI.

Matrices are torch float64 CUDA tensors viewed column-major: a logical
m x n matrix has strides (1, ld), exactly Mat's MAT<T> layout
(Mat-8.3.1/Base/__Matrix.h:141-146).  ``colmajor(m, n)`` makes one and
``as_colmajor(t)`` converts any tensor.  Every call goes through
libmatgpu.so; nothing here computes on the CPU.
"""
from __future__ import annotations

import ctypes as C

import torch

from ._lib import IrOpts, IrReport, MatGpuError, load

_F64 = torch.float64


def colmajor(m: int, n: int, dtype=_F64, device="cuda") -> torch.Tensor:
    """An uninitialised m x n column-major matrix (ld = m)."""
    return torch.empty((n, m), dtype=dtype, device=device).t()


def as_colmajor(t: torch.Tensor, dtype=_F64, device="cuda") -> torch.Tensor:
    """Copy of ``t`` (logical 2-D) in column-major layout on ``device``."""
    t = t.to(device=device, dtype=dtype)
    return t.t().contiguous().t()


def ld_of(t: torch.Tensor) -> int:
    if t.dim() != 2:
        raise ValueError("expected a 2-D matrix")
    if t.shape[0] > 1 and t.stride(0) != 1:
        raise ValueError("matrix must be column-major (stride(0) == 1); use as_colmajor()")
    if t.shape[1] <= 1:
        return max(1, t.shape[0])
    return t.stride(1)


def _ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


class Handle:
    """Owns an mg_handle_t bound to a CUDA stream (default: torch's current stream)."""

    def __init__(self, stream: torch.cuda.Stream | None = None):
        self.lib = load()
        s = stream if stream is not None else torch.cuda.current_stream()
        self._stream = s
        h = C.c_void_p()
        self.check(self.lib.mg_handle_create(C.byref(h), C.c_void_p(s.cuda_stream)), "mg_handle_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.mg_handle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> torch.cuda.Stream:
        return self._stream

    def check(self, status: int, what: str = ""):
        if status != 0:
            msg = ""
            if getattr(self, "h", None):
                msg = (self.lib.mg_get_last_error(self.h) or b"").decode(errors="replace")
            raise MatGpuError(status, f"{what}: {msg}" if what else msg)

    def launch_count(self) -> int:
        return int(self.lib.mg_launch_count(self.h))

    # ------------------------------------------------------------ generators
    def fill_uniform(self, A: torch.Tensor, seed: int, lo=-1.0, hi=1.0, rowmajor_stream=True):
        self.check(self.lib.mg_fill_uniform(self.h, _ptr(A), A.shape[0], A.shape[1], ld_of(A), seed,
                                            lo, hi, int(rowmajor_stream)), "mg_fill_uniform")
        return A

    def fill_normal(self, A: torch.Tensor, seed: int, rowmajor_stream=True):
        self.check(self.lib.mg_fill_normal(self.h, _ptr(A), A.shape[0], A.shape[1], ld_of(A), seed,
                                           int(rowmajor_stream)), "mg_fill_normal")
        return A

    # ------------------------------------------------------------------ GEMM
    def dgemm(self, A, B, C_=None, alpha=1.0, beta=0.0, transA=False, transB=False):
        """C = alpha op(A) op(B) + beta C (Mat's operator* when alpha=1, beta=0)."""
        m = A.shape[1] if transA else A.shape[0]
        k = A.shape[0] if transA else A.shape[1]
        n = B.shape[0] if transB else B.shape[1]
        kb = B.shape[1] if transB else B.shape[0]
        if k != kb:
            raise ValueError(f"inner dimensions differ: {k} vs {kb}")
        if C_ is None:
            C_ = colmajor(m, n, device=A.device)
            beta = 0.0
        self.check(self.lib.mg_dgemm(self.h, int(transA), int(transB), m, n, k, alpha, _ptr(A), ld_of(A),
                                     _ptr(B), ld_of(B), beta, _ptr(C_), ld_of(C_)), "mg_dgemm")
        return C_

    def sgemm(self, A, B, C_=None, alpha=1.0, beta=0.0, transA=False, transB=False):
        """fp32 C = alpha op(A) op(B) + beta C (SIMT FFMA)."""
        m = A.shape[1] if transA else A.shape[0]
        k = A.shape[0] if transA else A.shape[1]
        n = B.shape[0] if transB else B.shape[1]
        if C_ is None:
            C_ = colmajor(m, n, dtype=torch.float32, device=A.device)
            beta = 0.0
        self.check(self.lib.mg_sgemm(self.h, int(transA), int(transB), m, n, k, alpha, _ptr(A), ld_of(A), _ptr(B),
                                     ld_of(B), beta, _ptr(C_), ld_of(C_)), "mg_sgemm")
        return C_

    def sgemm_bf16x(self, A, B, C_=None, alpha=1.0, beta=0.0, nterms=3, ordered=False):
        """fp32 C = alpha A B + beta C on the BF16 tensor cores with `nterms` split
        terms; ordered: lower-order products first (more accurate, slower)."""
        m, k = A.shape
        n = B.shape[1]
        if C_ is None:
            C_ = colmajor(m, n, dtype=torch.float32, device=A.device)
            beta = 0.0
        self.check(self.lib.mg_sgemm_bf16x_ex(self.h, nterms, 1 if ordered else 0, m, n, k, alpha, _ptr(A), ld_of(A),
                                              _ptr(B), ld_of(B), beta, _ptr(C_), ld_of(C_)), "mg_sgemm_bf16x_ex")
        flag = C.c_int(0)
        self.check(self.lib.mg_bf16x_check_error(self.h, C.byref(flag)), "mg_bf16x_check_error")
        if flag.value:
            raise MatGpuError(flag.value, "split GEMM: a bounded device wait timed out")
        return C_

    # -------------------------------------------------------------------- LU
    def dgetrf(self, A: torch.Tensor, pos: torch.Tensor | None = None, check=True):
        """In-place Mat PLU of A (m x n, column-major). Returns (pos, info)."""
        m, n = A.shape
        if pos is None:
            pos = torch.empty(m, dtype=torch.int32, device=A.device)
        info = C.c_int(0)
        st = self.lib.mg_dgetrf(self.h, m, n, _ptr(A), ld_of(A), _ptr(pos), C.byref(info))
        if check and st not in (0, 4):
            self.check(st, "mg_dgetrf")
        return pos, info.value

    def dgetrs(self, LU: torch.Tensor, pos: torch.Tensor, B: torch.Tensor, X: torch.Tensor | None = None):
        n = LU.shape[0]
        nrhs = B.shape[1]
        if X is None:
            X = colmajor(n, nrhs, device=B.device)
        self.check(self.lib.mg_dgetrs(self.h, n, nrhs, _ptr(LU), ld_of(LU), _ptr(pos), _ptr(B), ld_of(B),
                                      _ptr(X), ld_of(X)), "mg_dgetrs")
        return X

    def dgesv(self, A: torch.Tensor, B: torch.Tensor, X: torch.Tensor | None = None):
        """Mat Solve_direct(A, B): X = A^-1 B, A untouched. Returns (X, info)."""
        n = A.shape[0]
        nrhs = B.shape[1]
        if X is None:
            X = colmajor(n, nrhs, device=B.device)
        info = C.c_int(0)
        st = self.lib.mg_dgesv(self.h, n, nrhs, _ptr(A), ld_of(A), _ptr(B), ld_of(B), _ptr(X), ld_of(X),
                               C.byref(info))
        if st not in (0, 4):
            self.check(st, "mg_dgesv")
        return X, info.value

    # ----------------------------------------------------------------- mixed
    def ddet(self, A: torch.Tensor) -> float:
        """Mat Det(A) (A untouched)."""
        d = C.c_double()
        self.check(self.lib.mg_ddet(self.h, A.shape[0], _ptr(A), ld_of(A), C.byref(d)), "mg_ddet")
        return d.value

    def dinv(self, A: torch.Tensor, Ainv: torch.Tensor | None = None):
        """Mat Inv(A) (A untouched). Returns (Ainv, info)."""
        n = A.shape[0]
        if Ainv is None:
            Ainv = colmajor(n, n, device=A.device)
        info = C.c_int(0)
        st = self.lib.mg_dinv(self.h, n, _ptr(A), ld_of(A), _ptr(Ainv), ld_of(Ainv), C.byref(info))
        if st not in (0, 4):
            self.check(st, "mg_dinv")
        return Ainv, info.value

    def sgetf2(self, A: torch.Tensor, pos: torch.Tensor | None = None, tournament: bool = False):
        """In-place fp32 panel LU of A (m x n, n <= 128, column-major), partial or
        tournament pivoting. Returns (pos, info)."""
        m, n = A.shape
        if pos is None:
            pos = torch.empty(m, dtype=torch.int32, device=A.device)
        info = C.c_int(0)
        st = self.lib.mg_sgetf2_ex(self.h, 1 if tournament else 0, m, n, _ptr(A), ld_of(A), _ptr(pos),
                                   C.byref(info))
        if st not in (0, 4):
            self.check(st, "mg_sgetf2")
        return pos, info.value

    def sgetrf(self, A: torch.Tensor, pos: torch.Tensor | None = None):
        """In-place fp32 blocked LU of A (n x n, column-major) as in the mixed solve. Returns (pos, info)."""
        n = A.shape[0]
        if pos is None:
            pos = torch.empty(n, dtype=torch.int32, device=A.device)
        info = C.c_int(0)
        st = self.lib.mg_sgetrf(self.h, n, _ptr(A), ld_of(A), _ptr(pos), C.byref(info))
        if st not in (0, 4):
            self.check(st, "mg_sgetrf")
        return pos, info.value

    def dresidual(self, A, X, B, R=None, mode=0):
        """R = B - A X: mode 0 the exact fixed-point integer residual, 1 FP64 FMA."""
        n, nrhs = B.shape
        if R is None:
            R = colmajor(n, nrhs, device=B.device)
        self.check(self.lib.mg_dresidual(self.h, n, nrhs, _ptr(A), ld_of(A), _ptr(X), ld_of(X), _ptr(B), ld_of(B),
                                         _ptr(R), ld_of(R), int(mode)), "mg_dresidual")
        return R

    def dsgesv_ir(self, A, B, X=None, tol=1e-14, max_iter=30, nterms=3, fallback=True, gmres=True, panel=0,
                  residual=0, spd=False, qr=False):
        """Mixed LU (fp32 + split-BF16) + FP64 refinement, GMRES-IR and the FP64
        fallback when refinement stalls; spd=True: the fp32 Cholesky form
        (mg_dsposv_ir). residual: 0 = the exact fixed-point integer residual,
        1 = FP64 FMA. Returns (X, report dict with the status)."""
        n = A.shape[0]
        nrhs = B.shape[1]
        if X is None:
            X = colmajor(n, nrhs, device=B.device)
        o = IrOpts(tol, max_iter, nterms, int(fallback), int(gmres), int(panel), int(residual))
        r = IrReport()
        name = "mg_dsqrsv_ir" if qr else "mg_dsposv_ir" if spd else "mg_dsgesv_ir"
        st = getattr(self.lib, name)(self.h, n, nrhs, _ptr(A), ld_of(A), _ptr(B), ld_of(B), _ptr(X), ld_of(X),
                                     C.byref(o), C.byref(r))
        if st not in (0, 6, 7):
            self.check(st, name)
        nh = min(32, r.iterations + 1)
        rep = dict(iterations=r.iterations, path=r.path, info=r.info, gmres_iterations=r.gmres_iterations,
                   backward_error=r.backward_error, anorm_inf=r.anorm_inf, factor_ms=r.factor_ms,
                   refine_ms=r.refine_ms, history=[r.history[i] for i in range(nh)],
                   pivot_growth=r.pivot_growth, status=st)
        return X, rep

    def dsposv_ir(self, A, B, X=None, **kw):
        """Mixed-precision SPD solve (fp32 Cholesky with split-BF16 updates + FP64 refinement)."""
        return self.dsgesv_ir(A, B, X, spd=True, **kw)

    def dsqrsv_ir(self, A, B, X=None, **kw):
        """Mixed-precision solve through Householder QR (fp32 QR with FP64 norms, split-BF16
        updates; FP64 refinement)."""
        return self.dsgesv_ir(A, B, X, qr=True, **kw)

    def sgeqrf(self, A):
        """In-place fp32 Householder QR of A (m x n, m >= n). Returns (tau float64, T blocks float32)."""
        m, n = A.shape
        tau = torch.empty(n, dtype=torch.float64, device=A.device)
        T = torch.empty(((n + 127) // 128) * 128 * 128, dtype=torch.float32, device=A.device)
        self.check(self.lib.mg_sgeqrf(self.h, m, n, _ptr(A), ld_of(A), _ptr(tau), _ptr(T)), "mg_sgeqrf")
        return tau, T

    # ------------------------------------------------------------- generators
    def gen_svd_matrix(self, A, seed, nrefl=64, sigma_min=1e-6):
        n = A.shape[0]
        self.check(self.lib.mg_gen_svd_matrix(self.h, n, _ptr(A), ld_of(A), seed, nrefl, sigma_min),
                   "mg_gen_svd_matrix")
        return A

    def gen_spd_gram(self, S, seed):
        n = S.shape[0]
        self.check(self.lib.mg_gen_spd_gram(self.h, n, _ptr(S), ld_of(S), seed), "mg_gen_spd_gram")
        return S

    # -------------------------------------------------------------- Cholesky
    def dpotrf(self, A: torch.Tensor, check=True):
        """In-place Mat LLT: lower triangle of A -> L, upper zeroed. Returns info."""
        n = A.shape[0]
        info = C.c_int(0)
        st = self.lib.mg_dpotrf(self.h, n, _ptr(A), ld_of(A), C.byref(info))
        if check and st not in (0, 5):
            self.check(st, "mg_dpotrf")
        return info.value

    def dlu(self, A: torch.Tensor) -> int:
        """In-place Mat LU without pivoting (square A): multipliers below the
        diagonal, U on and above. Returns info."""
        info = C.c_int(0)
        st = self.lib.mg_dlu(self.h, A.shape[0], _ptr(A), ld_of(A), C.byref(info))
        if st not in (0, 4):
            self.check(st, "mg_dlu")
        return info.value

    def dldlt(self, A: torch.Tensor, d: torch.Tensor | None = None):
        """In-place Mat LDLT: lower triangle of A -> L (upper zeroed); returns (d, info)."""
        n = A.shape[0]
        if d is None:
            d = torch.empty(n, dtype=torch.float64, device=A.device)
        info = C.c_int(0)
        st = self.lib.mg_dldlt(self.h, n, _ptr(A), ld_of(A), _ptr(d), C.byref(info))
        if st not in (0, 4):
            self.check(st, "mg_dldlt")
        return d, info.value

    def dtridiag81(self, A: torch.Tensor):
        """Mat-8.1 EVD_Q tridiagonalisation of the symmetric A (lower triangle
        read; reflectors left below its diagonal): returns (Q, d, e) with
        Q^T A Q = tridiag(e, d, e)."""
        n = A.shape[0]
        Q = colmajor(n, n, device=A.device)
        d = torch.empty(n, dtype=torch.float64, device=A.device)
        e = torch.empty(max(n - 1, 1), dtype=torch.float64, device=A.device)
        self.check(self.lib.mg_dtridiag81(self.h, n, _ptr(A), ld_of(A), _ptr(Q), ld_of(Q), _ptr(d), _ptr(e)),
                   "mg_dtridiag81")
        return Q, d, e[: n - 1]

    def devd_q(self, A: torch.Tensor, eps: float, E: torch.Tensor | None = None, Q: torch.Tensor | None = None):
        """Mat-8.1 EVD_Q(A, E, Q, eps, EVD_QR): returns (w, E, Q), A Q = Q E, E = diag(w)."""
        n = A.shape[0]
        E = colmajor(n, n, device=A.device) if E is None else E
        Q = colmajor(n, n, device=A.device) if Q is None else Q
        w = torch.empty(n, dtype=torch.float64, device=A.device)
        self.check(self.lib.mg_devd_q(self.h, n, _ptr(A), ld_of(A), float(eps), _ptr(E), ld_of(E), _ptr(Q),
                                      ld_of(Q), _ptr(w)), "mg_devd_q")
        return w, E, Q

    def spotrf(self, A: torch.Tensor, check=True):
        """In-place fp32 LLT: lower triangle of A -> L, upper zeroed. Returns info."""
        n = A.shape[0]
        info = C.c_int(0)
        st = self.lib.mg_spotrf(self.h, n, _ptr(A), ld_of(A), C.byref(info))
        if check and st not in (0, 5):
            self.check(st, "mg_spotrf")
        return info.value

    def dpotrs(self, L: torch.Tensor, B: torch.Tensor):
        """In place: B := (L L^T)^-1 B."""
        self.check(self.lib.mg_dpotrs(self.h, L.shape[0], B.shape[1], _ptr(L), ld_of(L), _ptr(B), ld_of(B)),
                   "mg_dpotrs")
        return B

    # -------------------------------------------------------------------- QR
    def dqr(self, A: torch.Tensor, Q: torch.Tensor | None = None, R: torch.Tensor | None = None):
        """Mat QR(A, Q, R, QR_Householder): full m x m Q and m x n R (A unchanged)."""
        m, n = A.shape
        if Q is None:
            Q = colmajor(m, m, device=A.device)
        if R is None:
            R = colmajor(m, n, device=A.device)
        self.check(self.lib.mg_dqr(self.h, m, n, _ptr(A), ld_of(A), _ptr(Q), ld_of(Q), _ptr(R), ld_of(R)),
                   "mg_dqr")
        return Q, R

    # -------------------------------------------------------------- adjoints
    def dpotrf_backward(self, L, Lbar, Abar=None):
        n = L.shape[0]
        if Abar is None:
            Abar = colmajor(n, n, device=L.device)
        self.check(self.lib.mg_dpotrf_backward(self.h, n, _ptr(L), ld_of(L), _ptr(Lbar), ld_of(Lbar), _ptr(Abar),
                                               ld_of(Abar)), "mg_dpotrf_backward")
        return Abar

    def spotrf_backward(self, L, Lbar, Abar=None):
        n = L.shape[0]
        if Abar is None:
            Abar = colmajor(n, n, dtype=torch.float32, device=L.device)
        self.check(self.lib.mg_spotrf_backward(self.h, n, _ptr(L), ld_of(L), _ptr(Lbar), ld_of(Lbar), _ptr(Abar),
                                               ld_of(Abar)), "mg_spotrf_backward")
        return Abar

    def dtrsm_backward(self, L, X, Xbar, Lbar, trans=False):
        """X = op(L)^-1 B. Returns Bbar; accumulates into the lower triangle of Lbar."""
        n, nrhs = X.shape
        Bbar = colmajor(n, nrhs, device=X.device)
        self.check(self.lib.mg_dtrsm_backward(self.h, int(trans), n, nrhs, _ptr(L), ld_of(L), _ptr(X), ld_of(X),
                                              _ptr(Xbar), ld_of(Xbar), _ptr(Bbar), ld_of(Bbar), _ptr(Lbar),
                                              ld_of(Lbar)), "mg_dtrsm_backward")
        return Bbar

    def dlogdet_chol(self, L) -> float:
        out = C.c_double()
        self.check(self.lib.mg_dlogdet_chol(self.h, L.shape[0], _ptr(L), ld_of(L), C.byref(out)), "mg_dlogdet_chol")
        return out.value

    def dlogdet_chol_backward(self, L, gbar, Lbar):
        self.check(self.lib.mg_dlogdet_chol_backward(self.h, L.shape[0], _ptr(L), ld_of(L), float(gbar), _ptr(Lbar),
                                                     ld_of(Lbar)), "mg_dlogdet_chol_backward")
        return Lbar

    def gen_rbf_kernel(self, X, ell, sigma2=1.0, jitter=1e-2, K=None):
        n = X.shape[0]
        if K is None:
            K = colmajor(n, n, device=X.device)
        self.check(self.lib.mg_gen_rbf_kernel(self.h, n, _ptr(X), ell, sigma2, jitter, _ptr(K), ld_of(K)),
                   "mg_gen_rbf_kernel")
        return K

    def gp_loss_grad(self, X, y, ell, sigma2=1.0, jitter=1e-2, want_kbar=False):
        n = X.shape[0]
        loss, dell = C.c_double(), C.c_double()
        Kb = colmajor(n, n, device=X.device) if want_kbar else None
        self.check(self.lib.mg_gp_loss_grad(self.h, n, _ptr(X), ell, sigma2, jitter, _ptr(y), C.byref(loss),
                                            C.byref(dell), _ptr(Kb), ld_of(Kb) if Kb is not None else n),
                   "mg_gp_loss_grad")
        return loss.value, dell.value, Kb

    def sgp_loss_grad(self, X, y, ell, sigma2=1.0, jitter=1e-2, want_kbar=False):
        """FP32 form of gp_loss_grad (X, y float32); loss and d/d ell summed in fp64."""
        n = X.shape[0]
        loss, dell = C.c_double(), C.c_double()
        Kb = colmajor(n, n, dtype=torch.float32, device=X.device) if want_kbar else None
        self.check(self.lib.mg_sgp_loss_grad(self.h, n, _ptr(X), ell, sigma2, jitter, _ptr(y), C.byref(loss),
                                             C.byref(dell), _ptr(Kb), ld_of(Kb) if Kb is not None else n),
                   "mg_sgp_loss_grad")
        return loss.value, dell.value, Kb

    # --------------------------------------------------------------- profile
    def profile(self, on: bool = True, only: str | None = None):
        """Per-phase CUDA-event timing on the library's streams (all phases, or
        only those named `only`)."""
        self.check(self.lib.mg_profile_only(self.h, (only or "").encode()), "mg_profile_only")
        self.check(self.lib.mg_profile_enable(self.h, int(on)), "mg_profile_enable")

    def profile_records(self) -> dict:
        out = {}
        for i in range(self.lib.mg_profile_count(self.h)):
            name = C.c_char_p()
            ms, fl, by = C.c_double(), C.c_double(), C.c_double()
            la = C.c_longlong()
            self.check(self.lib.mg_profile_get(self.h, i, C.byref(name), C.byref(ms), C.byref(la), C.byref(fl),
                                               C.byref(by)), "mg_profile_get")
            out[name.value.decode()] = dict(ms=ms.value, launches=la.value, flops=fl.value, bytes=by.value)
        return out

    def measure_fp64_peaks(self) -> tuple[float, float]:
        a, b = C.c_double(), C.c_double()
        self.check(self.lib.mg_measure_fp64_peaks(self.h, C.byref(a), C.byref(b)), "mg_measure_fp64_peaks")
        return a.value, b.value


def host_fill_uniform(rows: int, cols: int, seed: int, lo=-1.0, hi=1.0, rowmajor_stream=True):
    """Seeded uniform matrix on the host (numpy, column-major), bit-identical to fill_uniform."""
    import numpy as np
    a = np.empty((rows, cols), dtype=np.float64, order="F")
    load().mg_host_fill_uniform(a.ctypes.data, rows, cols, max(rows, 1), seed, lo, hi, int(rowmajor_stream))
    return a


def host_steqr81(d, e, eps: float):
    """Mat-8.1 EVD_Q's QR sweeps on the host (no GPU): eigenvalues of the
    tridiagonal (d, e) in Mat's order, and the number of plane rotations."""
    import numpy as np
    d = np.array(d, dtype=np.float64)
    e = np.ascontiguousarray(e, dtype=np.float64)
    rot = C.c_longlong(0)
    st = load().mg_dsteqr81_host(len(d), d.ctypes.data, e.ctypes.data if len(e) else None, float(eps), C.byref(rot))
    if st != 0:
        raise MatGpuError(st, "mg_dsteqr81_host")
    return d, rot.value


def host_fill_normal(rows: int, cols: int, seed: int, rowmajor_stream=True):
    """Seeded N(0,1) matrix on the host (numpy, column-major), bit-identical to fill_normal."""
    import numpy as np
    a = np.empty((rows, cols), dtype=np.float64, order="F")
    load().mg_host_fill_normal(a.ctypes.data, rows, cols, max(rows, 1), seed, int(rowmajor_stream))
    return a
