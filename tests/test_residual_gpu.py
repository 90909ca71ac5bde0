"""The residual R = B - A X of the mixed solves (mg_dresidual): the exact
fixed-point integer form (mode 0) against exact rational arithmetic and
against FP64 FMA (mode 1); non-finite inputs; the mixed solves with either
residual.  The reference has no residual of its own (Mat solves once, in
FP64: Mat-8.3.1/LU/__Solve_direct.h:70-142); the bound checked for mode 0 is
its own error model: every entry rounded once to 2^-63 of its row's (A) or
column's (X) largest power of two, exact products and sums, one rounding to
double and the FP64 subtraction."""
from fractions import Fraction

import numpy as np
import pytest
import torch

from mat_gb300.api import Handle, colmajor

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def handle():
    return Handle()


def _cm(a):
    """A column-major float64 CUDA tensor holding numpy array a."""
    t = colmajor(a.shape[0], a.shape[1])
    t.copy_(torch.from_numpy(np.ascontiguousarray(a)))
    return t


def _exact_residual(a, x, b):
    n, nrhs = b.shape
    r = np.empty((n, nrhs))
    for j in range(nrhs):
        xf = [Fraction(float(v)) for v in x[:, j]]
        for i in range(n):
            s = Fraction(float(b[i, j])) - sum(Fraction(float(a[i, k])) * xf[k] for k in range(n) if a[i, k] != 0)
            r[i, j] = float(s)
    return r


def _pow2_max(v):
    """2^e with e the exponent of the largest |v| (its power-of-two scale)."""
    m = np.abs(v).max()
    return 0.0 if m == 0 else 2.0 ** np.floor(np.log2(m))


@pytest.mark.parametrize("n,nrhs", [(67, 1), (130, 3)])
def test_integer_residual_matches_exact(handle, n, nrhs):
    rng = np.random.default_rng(n)
    a = rng.standard_normal((n, n))
    a *= 2.0 ** rng.integers(-30, 30, size=(n, 1))        # rows of very different scales
    a[3, :] = 0.0                                          # a zero row
    a[5, :7] = np.ldexp(rng.standard_normal(7), -1060)    # subnormals beside normal entries
    a[7, 1] = 1e300                                        # one entry dominating its row
    x = rng.standard_normal((n, nrhs)) * 2.0 ** rng.integers(-5, 5, size=(1, nrhs))
    b = a @ x + rng.standard_normal((n, nrhs)) * 1e-8      # a small residual: cancellation
    A, X, B = _cm(a), _cm(x), _cm(b)
    r0 = handle.dresidual(A, X, B, mode=0).cpu().numpy()
    r1 = handle.dresidual(A, X, B, mode=1).cpu().numpy()
    ex = _exact_residual(a, x, b)
    for j in range(nrhs):
        sx = _pow2_max(x[:, j])
        for i in range(n):
            sa = _pow2_max(a[i])
            # n entries each rounded to 2^-63 of its scale (of A's row / X's column,
            # products below 2^124 of the two scales), the dropped lowest digit
            # class, and the final roundings of the sum and of b - sum
            bound = n * 2.0 ** -58 * sa * sx * 4 + 2.0 ** -51 * (abs(ex[i, j]) + abs(b[i, j]))
            assert abs(r0[i, j] - ex[i, j]) <= bound, (i, j, r0[i, j], ex[i, j], bound)
    # and more accurate than the FP64 residual, relative to the scales
    sa = np.array([_pow2_max(a[i]) for i in range(n)])[:, None]
    sx = np.array([_pow2_max(x[:, j]) for j in range(nrhs)])[None, :]
    keep = (sa * sx) > 0
    e0 = (np.abs(r0 - ex)[keep] / (sa * sx)[keep]).max()
    e1 = (np.abs(r1 - ex)[keep] / (sa * sx)[keep]).max()
    assert e0 <= e1, (e0, e1)


@pytest.mark.parametrize("n,nrhs,ld", [(1000, 1, 1000), (2048, 4, 2051), (4097, 8, 4100), (3000, 5, 3000)])
def test_integer_residual_vs_fp64(handle, n, nrhs, ld):
    g = torch.Generator(device="cuda").manual_seed(n)
    A = torch.as_strided(torch.randn((n * ld,), generator=g, device="cuda", dtype=torch.float64), (n, n), (1, ld))
    X = torch.randn((nrhs, n), generator=g, device="cuda", dtype=torch.float64).t()
    B = (A @ X) + 1e-6 * torch.randn((nrhs, n), generator=g, device="cuda", dtype=torch.float64).t()
    B = B.t().contiguous().t()
    r0 = handle.dresidual(A, X, B, mode=0)
    r1 = handle.dresidual(A, X, B, mode=1)
    scale = (A.abs() @ X.abs()).max(0).values  # |A||X| per column
    d = ((r0 - r1).abs().max(0).values / scale).max().item()
    assert d < 4e-15, d
    if n * nrhs > 2048 * 4:
        return
    # an extended-precision reference on the host: mode 0 within its model
    a = A.cpu().numpy().astype(np.longdouble)
    x = X.cpu().numpy().astype(np.longdouble)
    ref = (B.cpu().numpy().astype(np.longdouble) - a @ x).astype(np.float64)
    e0 = (np.abs(r0.cpu().numpy() - ref).max(0) / scale.cpu().numpy()).max()
    e1 = (np.abs(r1.cpu().numpy() - ref).max(0) / scale.cpu().numpy()).max()
    if np.finfo(np.longdouble).nmant >= 63:  # a reference finer than FP64 on this host
        assert e0 <= max(2.0 * e1, 2e-17), (e0, e1)


def test_integer_residual_nonfinite(handle):
    n = 300
    rng = np.random.default_rng(0)
    a, x = rng.standard_normal((n, n)), rng.standard_normal((n, 2))
    b = a @ x
    a_nan = a.copy()
    a_nan[10, 20] = np.nan
    r = handle.dresidual(_cm(a_nan), _cm(x), _cm(b), mode=0).cpu().numpy()
    assert np.isnan(r[10]).all() and np.isfinite(np.delete(r, 10, axis=0)).all()  # FP64 taken: NaN in row 10 only
    x_inf = x.copy()
    x_inf[3, 1] = np.inf
    r = handle.dresidual(_cm(a), _cm(x_inf), _cm(b), mode=0).cpu().numpy()
    assert not np.isfinite(r).all()


@pytest.mark.parametrize("kind", ["lu", "spd", "qr"])
def test_mixed_solves_with_either_residual(handle, kind):
    n, nrhs = 2000, 3
    if kind == "spd":
        g = torch.Generator(device="cuda").manual_seed(5)
        pts = torch.rand((3, n), generator=g, device="cuda", dtype=torch.float64).t()
        A = handle.gen_rbf_kernel(pts, 0.2, 1.0, 1e-2)
    else:
        A = colmajor(n, n)
        handle.gen_svd_matrix(A, 3, nrefl=64, sigma_min=1e-6)
    B = colmajor(n, nrhs)
    handle.fill_normal(B, 11)
    res = {}
    for mode in (0, 1):
        X, rep = handle.dsgesv_ir(A, B, residual=mode, spd=kind == "spd", qr=kind == "qr")
        assert rep["status"] == 0 and rep["path"] == 0, rep
        r = B - A @ X
        eta = (r.abs().max(0).values / (A.abs().sum(1).max() * X.abs().max(0).values + B.abs().max(0).values)).max()
        assert eta.item() <= 1e-14, (mode, eta.item())
        res[mode] = (X, rep)
    # the two residuals steer refinement the same way
    assert abs(res[0][1]["iterations"] - res[1][1]["iterations"]) <= 1
    d = ((res[0][0] - res[1][0]).abs().max() / res[1][0].abs().max()).item()
    assert d < 1e-9, d
