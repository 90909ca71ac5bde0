"""mg_dgetrf_noalloc, the allocation-free LU entry point for callers that
cannot allocate device memory while they factor (memory owned by another
system's pool or budget, or no device-wide synchronisation allowed), checked
through the C ABI against mg_dgetrf on the same inputs, twice in a row: the
shared scratch array keeps the previous call's contents, so the second call
shows that everything that must start at zero is cleared.  Both entry points
run the same kernels in the same order, so factors and pivots must be equal
bit for bit.  Collected last so that a run stopping at the first failure has
already run every other test."""
import ctypes as C

import pytest
import torch

from mat_gb300 import _lib
from mat_gb300.api import Handle, colmajor

pytestmark = pytest.mark.gpu


def _both(lib, h, stream, A0):
    """Factors a copy of A0 with mg_dgetrf and with mg_dgetrf_noalloc."""
    m, n = A0.shape
    Aref, Anoa = A0.clone(), A0.clone()
    pref = torch.empty(m, dtype=torch.int32, device="cuda")
    pnoa = torch.full((m,), -7, dtype=torch.int32, device="cuda")
    info_ref, info_noa = C.c_int(-1), C.c_int(-1)
    st_ref = lib.mg_dgetrf(h.h, m, n, C.c_void_p(Aref.data_ptr()), m, C.c_void_p(pref.data_ptr()),
                           C.byref(info_ref))
    st_noa = lib.mg_dgetrf_noalloc(stream, m, n, C.c_void_p(Anoa.data_ptr()), m, C.c_void_p(pnoa.data_ptr()),
                                   C.byref(info_noa))
    torch.cuda.synchronize()
    return (st_ref, info_ref.value, Aref, pref), (st_noa, info_noa.value, Anoa, pnoa)


def _setup():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return _lib.load(), Handle(), C.c_void_p(torch.cuda.current_stream().cuda_stream)


@pytest.mark.parametrize("m,n", [(61, 61), (1000, 1000), (1000, 300), (40000, 80)])
def test_noalloc_lu_matches_dgetrf_twice(m, n):
    lib, h, stream = _setup()
    for seed in (1, 2):  # two calls in a row on different inputs
        A0 = colmajor(m, n)
        h.fill_normal(A0, seed)
        (st_r, info_r, Ar, pr), (st_n, info_n, An, pn) = _both(lib, h, stream, A0)
        assert st_r == 0 and st_n == 0 and info_n == info_r == 0
        assert torch.equal(pn, pr)
        assert torch.equal(An, Ar)


def test_noalloc_singular_then_regular():
    """An exactly singular input reports MG_SINGULAR and the same info as
    mg_dgetrf; the next call on a regular input starts from clean status words."""
    lib, h, stream = _setup()
    n = 300
    A0 = colmajor(n, n)
    h.fill_normal(A0, 3)
    A0[:, 150] = 0.0  # column 151 (1-based) is zero: that pivot is exactly zero
    (st_r, info_r, Ar, pr), (st_n, info_n, An, pn) = _both(lib, h, stream, A0)
    assert st_r == st_n == 4  # MG_SINGULAR
    assert info_n == info_r == 151
    assert torch.equal(pn, pr) and torch.equal(An, Ar)
    h.fill_normal(A0, 4)
    (st_r, info_r, Ar, pr), (st_n, info_n, An, pn) = _both(lib, h, stream, A0)
    assert st_r == st_n == 0 and info_n == info_r == 0
    assert torch.equal(pn, pr) and torch.equal(An, Ar)


def test_noalloc_rejects_oversize():
    lib, h, stream = _setup()
    # beyond the fixed capacity (m > 65536) and, at width 90, beyond what one
    # unblocked panel can hold in the SMs' shared memory: both refused before
    # anything is launched (real buffers all the same, so nothing could fault)
    for m, n in ((70000, 10), (60000, 90)):
        A = torch.full((n, m), 1.0, dtype=torch.float64, device="cuda")
        pos = torch.full((m,), -7, dtype=torch.int32, device="cuda")
        st = lib.mg_dgetrf_noalloc(stream, m, n, C.c_void_p(A.data_ptr()), m, C.c_void_p(pos.data_ptr()), None)
        torch.cuda.synchronize()
        assert st == 9  # MG_ERR_UNSUPPORTED
        assert bool((pos == -7).all()) and bool((A == 1.0).all())  # nothing was launched
