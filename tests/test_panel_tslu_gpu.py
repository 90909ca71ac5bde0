"""Tournament pivoting in the FP32 panel of the mixed LU (mg_sgetf2_ex with
MG_PANEL_TOURNAMENT), against a restatement of the algorithm with exactly
rounded fp32 arithmetic (emulated in float64: the product of two fp32
values is exact there; the rare double rounding of the emulation aside,
the factors match bit for bit and the pivots exactly).

The panel's rows are dealt to the 16 CTAs of a cluster in contiguous runs
of RPC = 256 * ceil(R / 4096) rows; thread t of CTA q holds the positions
q * RPC + k * 256 + t, so warp w holds {q * RPC + k * 256 + 32 w + l}.  Per
16-column sub-panel the pivots come from a reduction tree of partial-pivoting
eliminations (first largest |a| per column, the smaller position on ties;
l = a * (1 / p), a := fma(l, -p, a)), each level passing on the rows it
picked as they were when the sub-panel started: each warp over its rows at
or below the sub-panel's diagonal, each CTA over its 8 warps' picks, each
pair of CTAs (2w, 2w+1) over their picks, then all 8 pairs' picks, whose
pick order is the pivot order.  Pivot c is swapped to position cs0 + c, in
order, and the sub-panel eliminated without further pivoting, right-looking
over the panel's columns.

The mixed solve with tournament panels reaches FP64 backward error within
the refinement budget, with its pivot growth reported and bounded.
"""
import numpy as np
import pytest
import torch

from mat_gb300.api import as_colmajor, colmajor

pytestmark = pytest.mark.gpu
F32 = np.float32


def r32(x):
    return np.asarray(x, dtype=np.float64).astype(F32).astype(np.float64)


def eliminate_pick(U, P, sw):
    """Partial-pivoting elimination of the rows U (positions P) over sw
    columns; returns per column the picked position, or -1."""
    U = U.copy()
    avail = np.ones(len(P), bool)
    picks = []
    for c in range(sw):
        col = np.abs(U[:, c])
        col = np.where(avail & ~np.isnan(col), col, -1.0)
        if len(col) == 0 or not col.max() > 0:
            picks.append(-1)
            continue
        idx = np.flatnonzero(col == col.max())
        k = idx[np.argmin(P[idx])]
        avail[k] = False
        picks.append(int(P[k]))
        prow = U[k].copy()
        inv = F32(1.0) / F32(prow[c])
        l = r32(U[avail, c].astype(F32) * inv)
        U[np.ix_(avail, np.arange(c + 1, sw))] = r32(U[avail, c + 1:sw] - np.outer(l, prow[c + 1:sw]))
    return picks


def tslu_restated(a32: np.ndarray):
    a = a32.astype(np.float64)
    m, w = a.shape
    R = m
    rpt = -(-R // (16 * 256))
    rpc = 256 * rpt
    perm = np.arange(m)
    info = 0
    for cs0 in range(0, w, 16):
        sw = min(16, w - cs0)
        S0 = a[:, cs0:cs0 + sw].copy()

        def level(P):
            P = np.array(sorted(set(int(x) for x in P if x >= 0)), dtype=np.int64)
            return eliminate_pick(S0[P], P, sw) if len(P) else [-1] * sw

        cta_picks = []
        for q in range(16):
            warp_picks = []
            for wv in range(8):
                P = [q * rpc + k * 256 + 32 * wv + l for k in range(rpt) for l in range(32)]
                P = [p for p in P if cs0 <= p < R]
                warp_picks += level(P)
            cta_picks.append(level(warp_picks))
        pair_picks = []
        for g in range(8):
            pair_picks += level(cta_picks[2 * g] + cta_picks[2 * g + 1])
        win = level(pair_picks)
        where = np.arange(m)  # current position of the row that started at each position
        rowat = np.arange(m)
        for c in range(sw):
            cabs = cs0 + c
            if win[c] < 0:
                info = info or cabs + 1
                continue
            cur = where[win[c]]
            if cur != cabs:
                a[[cabs, cur], :] = a[[cur, cabs], :]
                perm[[cabs, cur]] = perm[[cur, cabs]]
                ra, rb = rowat[cabs], rowat[cur]
                rowat[cabs], rowat[cur] = rb, ra
                where[ra], where[rb] = cur, cabs
        for c in range(sw):
            cabs = cs0 + c
            p = a[cabs, cabs]
            if p == 0:
                continue
            inv = F32(1.0) / F32(p)
            l = r32(a[cabs + 1:, cabs].astype(F32) * inv)
            a[cabs + 1:, cabs] = l
            a[cabs + 1:, cabs + 1:] = r32(a[cabs + 1:, cabs + 1:] - np.outer(l, a[cabs, cabs + 1:]))
    return a.astype(F32), perm, info


def run_panel(handle, a, tournament=True):
    A = as_colmajor(torch.from_numpy(a), dtype=torch.float32)
    pos, info = handle.sgetf2(A, tournament=tournament)
    torch.cuda.synchronize()
    return A.cpu().numpy(), pos.cpu().numpy(), info


@pytest.mark.parametrize("m,n", [(300, 128), (700, 40), (3000, 77), (4096, 128), (9000, 101), (16384, 128)])
def test_tournament_panel_matches_restatement(handle, m, n):
    rng = np.random.default_rng(m * 7 + n)
    a = rng.standard_normal((m, n)).astype(F32)
    got, pos, info = run_panel(handle, a)
    ref, perm, rinfo = tslu_restated(a)
    assert info == rinfo == 0
    np.testing.assert_array_equal(pos, perm)
    diff = np.abs(got.astype(np.float64) - ref.astype(np.float64))
    assert diff.max() <= 1e-5 * np.abs(ref).max(), diff.max()
    assert (diff != 0).mean() < 1e-4
    # and it is an LU factorization of the permuted panel
    L = np.tril(got.astype(np.float64), -1)[:, :n] + np.eye(m, n)
    U = np.triu(got.astype(np.float64))[:n, :]
    res = np.abs(a.astype(np.float64)[pos] - L @ U).max() / np.abs(a).max()
    assert res < 1e-5, res


def test_tournament_panel_zero_column(handle):
    m, n = 6000, 96
    rng = np.random.default_rng(9)
    a = rng.standard_normal((m, n)).astype(F32)
    a[:, 40] = 0.0  # exactly zero column: info 41, left unscaled
    got, pos, info = run_panel(handle, a)
    ref, perm, rinfo = tslu_restated(a)
    assert info == rinfo == 41
    np.testing.assert_array_equal(pos, perm)
    diff = np.abs(got.astype(np.float64) - ref.astype(np.float64))
    assert diff.max() <= 1e-5 * np.abs(ref).max()


def backward_error(a, x, b):
    r = b - a @ x
    return (np.abs(r).max(0) / (np.abs(a).sum(1).max() * np.abs(x).max(0) + np.abs(b).max(0))).max()


@pytest.mark.parametrize("n", [300, 1024, 2500, 4096])
def test_mixed_solve_with_tournament_panels(handle, n):
    A = colmajor(n, n)
    handle.gen_svd_matrix(A, 3, nrefl=64, sigma_min=1e-6)
    B = colmajor(n, 4)
    handle.fill_normal(B, 11)
    X, rep = handle.dsgesv_ir(A, B, panel=2, gmres=False, fallback=False)
    torch.cuda.synchronize()
    assert rep["status"] == 0 and rep["path"] == 0 and rep["iterations"] <= 4, rep
    assert backward_error(A.cpu().numpy(), X.cpu().numpy(), B.cpu().numpy()) <= 1e-14
    assert rep["pivot_growth"] < 100.0, rep["pivot_growth"]
