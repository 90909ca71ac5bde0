"""Mat call sites compiled against include/mat_gpu.hpp (the drop-in for
Mat.h) and linked to libmatgpu.so; results compared with the oracle
(the restatement of Mat-8.3.1 that is bit-identical to its AVX-512 build)."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from mat_gb300 import LIB_PATH
from mat_gb300.api import host_fill_normal, host_fill_uniform
from oracle.api import restatement

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def outputs(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    d = tmp_path_factory.mktemp("dropin")
    exe = d / "dropin"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", str(ROOT / "include"), str(ROOT / "tests/cpp/dropin_main.cpp"),
                    "-L", str(LIB_PATH.parent), "-lmatgpu", f"-Wl,-rpath,{LIB_PATH.parent}", "-o", str(exe)],
                   check=True)
    r = subprocess.run([str(exe), str(d)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return d


def load(d, name, shape, dtype=np.float64):
    a = np.fromfile(d / f"{name}.bin", dtype=dtype)
    return a.reshape(shape[::-1]).T if len(shape) == 2 else a


def test_operator_star_bit_identical(outputs):
    a = host_fill_uniform(150, 130, 0)
    b = host_fill_uniform(130, 170, 1)
    assert np.array_equal(load(outputs, "gemm", (150, 170)), restatement().dgemm(a, b))


def test_plu_bit_identical(outputs):
    g = host_fill_normal(300, 300, 2)
    pos, L, U = restatement().plu(g)
    assert np.array_equal(load(outputs, "plu_pos", (300,), np.int32), pos)
    assert np.array_equal(load(outputs, "plu_L", (300, 300)), L)
    assert np.array_equal(load(outputs, "plu_U", (300, 300)), U)


def test_lu_without_pivoting(outputs):
    a = host_fill_normal(200, 200, 4)
    a[np.diag_indices(200)] += 200.0
    L, U = restatement().lu(a)
    assert np.array_equal(load(outputs, "lu_L", (200, 200)), L)
    assert np.array_equal(load(outputs, "lu_U", (200, 200)), U)


def test_solve_and_det(outputs):
    g = host_fill_normal(300, 300, 2)
    b = host_fill_normal(300, 3, 3)
    assert np.array_equal(load(outputs, "solve", (300, 3)), restatement().solve(g, b))
    bw = host_fill_normal(300, 10, 8)
    assert np.array_equal(load(outputs, "solve_wide", (300, 10)), restatement().solve(g, bw))
    xm = load(outputs, "solve_mixed", (300, 3))
    r = b - g @ xm
    assert (np.abs(r).max(0) / (np.abs(g).sum(1).max() * np.abs(xm).max(0) + np.abs(b).max(0))).max() <= 1e-14
    det = load(outputs, "det", (1,))[0]
    assert det == restatement().det(g)
    assert np.array_equal(load(outputs, "inv", (300, 300)), restatement().inv(g))


def test_llt_bit_identical(outputs):
    s = load(outputs, "spd", (200, 200))
    assert np.array_equal(load(outputs, "llt", (200, 200)), restatement().llt(np.asfortranarray(s)))
    L, D = restatement().ldlt(np.asfortranarray(s))
    assert np.array_equal(load(outputs, "ldlt_L", (200, 200)), L)
    assert np.array_equal(load(outputs, "ldlt_D", (200, 200)), D)


def test_qr_bit_identical(outputs):
    a = host_fill_normal(300, 200, 7)
    q, r = restatement().qr(a)
    assert np.array_equal(load(outputs, "qr_Q", (300, 300)), q)
    assert np.array_equal(load(outputs, "qr_R", (300, 200)), r)


def test_evd_q_bit_identical(outputs):
    """EVD_Q(A, E, Q, eps, EVD_QR) through the drop-in header, on W + W^T
    (W the 200 x 200 seed-4 normal matrix, its leading 150 x 150 block)."""
    w = host_fill_normal(200, 200, 4)[:150, :150]
    a = np.asfortranarray(w + w.T)
    w0, q0 = restatement().evd_q81(a, 1e-10)
    assert np.array_equal(load(outputs, "evd_E", (150, 150)), np.diag(w0))
    assert np.array_equal(load(outputs, "evd_Q", (150, 150)), q0)


def test_float_operator_star(outputs):
    a = host_fill_uniform(150, 130, 0).reshape(-1, order="F")[:70 * 50].reshape(70, 50, order="F")
    b = host_fill_uniform(130, 170, 1).reshape(-1, order="F")[:50 * 60].reshape(50, 60, order="F")
    ref = a.astype(np.float32).astype(np.float64) @ b.astype(np.float32).astype(np.float64)
    got = load(outputs, "sgemm", (70, 60), np.float32).astype(np.float64)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 2e-6
