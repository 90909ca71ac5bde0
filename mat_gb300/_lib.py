"""ctypes binding of libmatgpu.so (the C ABI declared in include/mat_gpu.h).

The library is loaded from the package directory.  There is no CPU fallback:
if the library is missing, import fails with the build instruction, and the
compute calls return MG_ERR_CUDA when no CUDA device is present.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libmatgpu.so"

MG_STATUS = {
    0: "MG_OK", 1: "MG_ERR_ARG", 2: "MG_ERR_CUDA", 3: "MG_ERR_ALLOC", 4: "MG_SINGULAR",
    5: "MG_NOT_SPD", 6: "MG_IR_STALLED", 7: "MG_FALLBACK_USED", 8: "MG_TIMEOUT",
    9: "MG_ERR_UNSUPPORTED",
    10: "MG_NOT_CONVERGED",
}

vp = C.c_void_p
i32 = C.c_int
u64 = C.c_uint64
f64 = C.c_double
f32 = C.c_float
pi32 = C.POINTER(C.c_int)
pf64 = C.POINTER(C.c_double)


class IrOpts(C.Structure):
    _fields_ = [("tol", C.c_double), ("max_iter", C.c_int), ("nterms", C.c_int), ("fallback", C.c_int),
                ("gmres", C.c_int), ("panel", C.c_int), ("residual", C.c_int)]


class IrReport(C.Structure):
    _fields_ = [("iterations", C.c_int), ("path", C.c_int), ("info", C.c_int), ("gmres_iterations", C.c_int),
                ("backward_error", C.c_double), ("anorm_inf", C.c_double), ("factor_ms", C.c_double),
                ("refine_ms", C.c_double), ("history", C.c_double * 32), ("pivot_growth", C.c_double)]

# name -> (restype, argtypes); every symbol here is declared in include/mat_gpu.h
SIGNATURES: dict[str, tuple] = {
    "mg_handle_create": (i32, [C.POINTER(vp), vp]),
    "mg_handle_destroy": (i32, [vp]),
    "mg_set_stream": (i32, [vp, vp]),
    "mg_synchronize": (i32, [vp]),
    "mg_status_string": (C.c_char_p, [i32]),
    "mg_get_last_error": (C.c_char_p, [vp]),
    "mg_launch_count": (u64, [vp]),
    "mg_device_malloc": (i32, [C.POINTER(vp), C.c_size_t]),
    "mg_device_free": (i32, [vp]),
    "mg_host_malloc_pinned": (i32, [C.POINTER(vp), C.c_size_t]),
    "mg_host_free_pinned": (i32, [vp]),
    "mg_memcpy": (i32, [vp, vp, vp, C.c_size_t, i32]),
    "mg_host_fill_uniform": (None, [vp, i32, i32, i32, u64, f64, f64, i32]),
    "mg_host_fill_normal": (None, [vp, i32, i32, i32, u64, i32]),
    "mg_fill_uniform": (i32, [vp, vp, i32, i32, i32, u64, f64, f64, i32]),
    "mg_fill_normal": (i32, [vp, vp, i32, i32, i32, u64, i32]),
    "mg_dgemm": (i32, [vp, i32, i32, i32, i32, i32, f64, vp, i32, vp, i32, f64, vp, i32]),
    "mg_sgemm": (i32, [vp, i32, i32, i32, i32, i32, f32, vp, i32, vp, i32, f32, vp, i32]),
    "mg_measure_fp64_peaks": (i32, [vp, pf64, pf64]),
    "mg_selftest_bounded_wait": (i32, [vp, i32, i32, C.c_uint]),
    "mg_dgetrf": (i32, [vp, i32, i32, vp, i32, vp, pi32]),
    "mg_dgetrf_noalloc": (i32, [vp, i32, i32, vp, i32, vp, pi32]),
    "mg_sgetf2": (i32, [vp, i32, i32, vp, i32, vp, pi32]),
    "mg_sgetf2_ex": (i32, [vp, i32, i32, i32, vp, i32, vp, pi32]),
    "mg_ddet": (i32, [vp, i32, vp, i32, pf64]),
    "mg_dinv": (i32, [vp, i32, vp, i32, vp, i32, pi32]),
    "mg_dldlt": (i32, [vp, i32, vp, i32, vp, pi32]),
    "mg_dlu": (i32, [vp, i32, vp, i32, pi32]),
    "mg_dtridiag81": (i32, [vp, i32, vp, i32, vp, i32, vp, vp]),
    "mg_devd_q": (i32, [vp, i32, vp, i32, f64, vp, i32, vp, i32, vp]),
    "mg_dsteqr81_host": (i32, [i32, vp, vp, f64, C.POINTER(C.c_longlong)]),
    "mg_sgetrf": (i32, [vp, i32, vp, i32, vp, pi32]),
    "mg_dgetrs": (i32, [vp, i32, i32, vp, i32, vp, vp, i32, vp, i32]),
    "mg_dgesv": (i32, [vp, i32, i32, vp, i32, vp, i32, vp, i32, pi32]),
    "mg_sgemm_bf16x": (i32, [vp, i32, i32, i32, i32, f32, vp, i32, vp, i32, f32, vp, i32]),
    "mg_sgemm_bf16x_ex": (i32, [vp, i32, i32, i32, i32, i32, f32, vp, i32, vp, i32, f32, vp, i32]),
    "mg_bf16x_check_error": (i32, [vp, pi32]),
    "mg_dresidual": (i32, [vp, i32, i32, vp, i32, vp, i32, vp, i32, vp, i32, i32]),
    "mg_dsgesv_ir": (i32, [vp, i32, i32, vp, i32, vp, i32, vp, i32, C.POINTER(IrOpts), C.POINTER(IrReport)]),
    "mg_dsposv_ir": (i32, [vp, i32, i32, vp, i32, vp, i32, vp, i32, C.POINTER(IrOpts), C.POINTER(IrReport)]),
    "mg_dsqrsv_ir": (i32, [vp, i32, i32, vp, i32, vp, i32, vp, i32, C.POINTER(IrOpts), C.POINTER(IrReport)]),
    "mg_sgeqrf": (i32, [vp, i32, i32, vp, i32, vp, vp]),
    "mg_gen_svd_matrix": (i32, [vp, i32, vp, i32, u64, i32, f64]),
    "mg_gen_spd_gram": (i32, [vp, i32, vp, i32, u64]),
    "mg_profile_enable": (i32, [vp, i32]),
    "mg_profile_only": (i32, [vp, C.c_char_p]),
    "mg_profile_count": (i32, [vp]),
    "mg_profile_get": (i32, [vp, i32, C.POINTER(C.c_char_p), pf64, C.POINTER(C.c_longlong), pf64, pf64]),
    "mg_dpotrf": (i32, [vp, i32, vp, i32, pi32]),
    "mg_dpotrs": (i32, [vp, i32, i32, vp, i32, vp, i32]),
    "mg_spotrf": (i32, [vp, i32, vp, i32, pi32]),
    "mg_dqr": (i32, [vp, i32, i32, vp, i32, vp, i32, vp, i32]),
    "mg_dgeqrf": (i32, [vp, i32, i32, vp, i32, vp, vp]),
    "mg_dpotrf_backward": (i32, [vp, i32, vp, i32, vp, i32, vp, i32]),
    "mg_spotrf_backward": (i32, [vp, i32, vp, i32, vp, i32, vp, i32]),
    "mg_dtrsm_backward": (i32, [vp, i32, i32, i32, vp, i32, vp, i32, vp, i32, vp, i32, vp, i32]),
    "mg_dlogdet_chol": (i32, [vp, i32, vp, i32, pf64]),
    "mg_dlogdet_chol_backward": (i32, [vp, i32, vp, i32, f64, vp, i32]),
    "mg_gen_rbf_kernel": (i32, [vp, i32, vp, f64, f64, f64, vp, i32]),
    "mg_gp_loss_grad": (i32, [vp, i32, vp, f64, f64, f64, vp, pf64, pf64, vp, i32]),
    "mg_sgp_loss_grad": (i32, [vp, i32, vp, f32, f32, f32, vp, pf64, pf64, vp, i32]),
}

_lib = None


def load() -> C.CDLL:
    """Loads libmatgpu.so and declares every exported signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"` "
            "(or python mat_gb300/build.py)")
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class MatGpuError(RuntimeError):
    def __init__(self, status: int, msg: str = ""):
        self.status = status
        self.name = MG_STATUS.get(status, str(status))
        super().__init__(f"{self.name}: {msg}" if msg else self.name)
