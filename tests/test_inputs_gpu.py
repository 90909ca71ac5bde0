"""The GPU generator of the benchmark matrix A = Q1 diag(sigma) Q2
(mg_gen_svd_matrix) against the oracle's host restatement, bit for bit, up to
the benchmark size n = 16384 (whose digest the reference golden fixtures also
record); so the CPU baselines and the reference arm solve exactly the
system the GPU solves."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest
import torch

from mat_gb300.api import colmajor
from oracle.api import gen_svd_matrix, host_fill_normal

pytestmark = pytest.mark.gpu
G = Path(__file__).resolve().parent / "golden"
META = json.loads((G / "golden.json").read_text())["cases"]


def sha(a):
    return hashlib.sha256(np.asfortranarray(a).tobytes(order="F")).hexdigest()


@pytest.mark.parametrize("n,seed,nrefl,smin", [(1, 3, 64, 1e-6), (97, 1, 8, 1e-3), (300, 3, 64, 1e-6),
                                               (1000, 5, 64, 1e-6), (2048, 3, 64, 1e-10)])
def test_gpu_generator_equals_oracle(handle, n, seed, nrefl, smin):
    A = colmajor(n, n)
    handle.gen_svd_matrix(A, seed, nrefl=nrefl, sigma_min=smin)
    torch.cuda.synchronize()
    assert np.array_equal(A.cpu().numpy(), gen_svd_matrix(n, seed, nrefl, smin))


def test_gpu_generator_benchmark_size(handle):
    n = 16384
    A = colmajor(n, n)
    handle.gen_svd_matrix(A, 3, nrefl=64, sigma_min=1e-6)
    B = colmajor(n, 4)
    handle.fill_normal(B, 11)
    torch.cuda.synchronize()
    hA = gen_svd_matrix(n, 3, 64, 1e-6)
    assert torch.equal(torch.from_numpy(hA).to("cuda"), A)
    assert torch.equal(torch.from_numpy(host_fill_normal(n, 4, 11)).to("cuda"), B)
    case = META.get("solve_svd_16384_4")
    if case is not None:
        assert sha(hA) == case["sha256_A"]
