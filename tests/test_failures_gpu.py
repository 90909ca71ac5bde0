"""Failure paths, made to happen deterministically and without faulting the
GPU.  Mat reports nothing (a zero pivot is a silent break,
Mat-8.3.1/LU/__PLU.h:68-71; a non-SPD input gives NaN, LU/__LLT.h:7); the
library returns status codes instead:

* every device-side wait is bounded: mg_selftest_bounded_wait runs the
  library's grid barrier (a cooperative launch in which one CTA never
  arrives) and its mbarrier wait (a phase nothing completes) with a small
  poll budget; the call returns MG_TIMEOUT and the next normal call on the
  same handle succeeds;
* refinement that cannot converge (condition 1e12, far beyond what an FP32
  factorization can refine) stalls; with the FP64 fallback on (and GMRES-IR
  off), the solve reports MG_FALLBACK_USED and path 2 and still reaches
  1e-14, with it off it reports MG_IR_STALLED."""
import numpy as np
import pytest
import torch

from mat_gb300.api import colmajor

pytestmark = pytest.mark.gpu

MG_OK, MG_IR_STALLED, MG_FALLBACK_USED, MG_TIMEOUT = 0, 6, 7, 8


def _small_solve_ok(handle):
    A = colmajor(300, 300)
    handle.fill_normal(A, 1)
    B = colmajor(300, 2)
    handle.fill_normal(B, 2)
    X, info = handle.dgesv(A, B)
    torch.cuda.synchronize()
    r = (B - A @ X).abs().max().item()
    assert info == 0 and r < 1e-10


@pytest.mark.parametrize("kind", [0, 1])
def test_bounded_wait_runs_out_and_handle_recovers(handle, kind):
    lib = handle.lib
    # every CTA arrives: the wait completes
    assert lib.mg_selftest_bounded_wait(handle.h, kind, -1, 4096) == MG_OK
    # one CTA withholds its arrival (kind 0) / nothing completes the phase (kind 1)
    assert lib.mg_selftest_bounded_wait(handle.h, kind, 3, 4096) == MG_TIMEOUT
    assert b"ran out" in lib.mg_get_last_error(handle.h)
    # the context and the handle are still usable
    _small_solve_ok(handle)
    assert lib.mg_selftest_bounded_wait(handle.h, kind, -1, 4096) == MG_OK


def test_selftest_rejects_bad_arguments(handle):
    lib = handle.lib
    assert lib.mg_selftest_bounded_wait(handle.h, 2, -1, 100) == 1
    assert lib.mg_selftest_bounded_wait(handle.h, 0, 8, 100) == 1
    assert lib.mg_selftest_bounded_wait(handle.h, 0, -1, 0) == 1


def backward_error(a, x, b):
    r = b - a @ x
    return (np.abs(r).max(0) / (np.abs(a).sum(1).max() * np.abs(x).max(0) + np.abs(b).max(0))).max()


def test_refinement_stall_falls_back_to_fp64(handle):
    n = 1024
    A = colmajor(n, n)
    handle.gen_svd_matrix(A, 5, nrefl=64, sigma_min=1e-12)
    B = colmajor(n, 2)
    handle.fill_normal(B, 12)
    X, rep = handle.dsgesv_ir(A, B, gmres=False)
    torch.cuda.synchronize()
    assert rep["status"] == MG_FALLBACK_USED and rep["path"] == 2, rep
    assert backward_error(A.cpu().numpy(), X.cpu().numpy(), B.cpu().numpy()) <= 1e-14
    X2, rep2 = handle.dsgesv_ir(A, B, gmres=False, fallback=False)
    torch.cuda.synchronize()
    assert rep2["status"] == MG_IR_STALLED and rep2["path"] == 0, rep2
    assert rep2["backward_error"] > 1e-14
