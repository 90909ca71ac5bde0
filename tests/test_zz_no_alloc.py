"""mg_dgetrf_noalloc, the allocation-free LU entry point for callers that
cannot allocate device memory while they factor (memory owned by another
system's pool or budget, or no device-wide synchronisation allowed), checked
through the C ABI against mg_dgetrf on the same inputs, twice in a row: the
shared scratch array keeps the previous call's contents, so the second call
shows that everything that must start at zero is cleared.  Collected last so
that a run stopping at the first failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest
import torch

from mat_gb300 import _lib
from mat_gb300.api import Handle, colmajor

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [61, 1000])
def test_noalloc_lu_matches_dgetrf_twice(n):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = _lib.load()
    h = Handle()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for seed in (1, 2):  # two calls in a row on different inputs
        A0 = colmajor(n, n)
        h.fill_normal(A0, seed)
        Aref, Anoa = A0.clone(), A0.clone()
        pref = torch.empty(n, dtype=torch.int32, device="cuda")
        pnoa = torch.full((n,), -7, dtype=torch.int32, device="cuda")
        info_ref, info_noa = C.c_int(-1), C.c_int(-1)
        assert lib.mg_dgetrf(h.h, n, n, C.c_void_p(Aref.data_ptr()), n, C.c_void_p(pref.data_ptr()),
                             C.byref(info_ref)) == 0
        st = lib.mg_dgetrf_noalloc(stream, n, n, C.c_void_p(Anoa.data_ptr()), n, C.c_void_p(pnoa.data_ptr()),
                                   C.byref(info_noa))
        torch.cuda.synchronize()
        assert st == 0 and info_noa.value == info_ref.value == 0
        # identical pivots; factors within the LU tests' 1e-13 (bit-identical in practice)
        assert torch.equal(pnoa, pref)
        diff = (Anoa - Aref).norm().item() / Aref.norm().item()
        assert diff <= 1e-13


def test_noalloc_rejects_oversize():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = _lib.load()
    # beyond the fixed capacity: refused before touching memory
    st = lib.mg_dgetrf_noalloc(None, 70000, 10, C.c_void_p(16), 70000, C.c_void_p(16), None)
    assert st == 9  # MG_ERR_UNSUPPORTED
