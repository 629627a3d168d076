"""Failure handling, injected from the host (no GPU fault is provoked).

The reference maps LAPACK failures of a window (info != 0 from dsygvd/dsygvx, e.g. an overlap
that is not positive definite) to RuntimeError (src/lrft_cpp.cpp:94,110).  Here:

* a NaN in one window's H_W, written through lres_set_windows: the pass returns LRES_ENUMERIC
  with status bit 1 in out[2] on both routes and both precisions; that window's sums are not
  finite and every other window's sums equal those of the clean pass bit for bit;
* an overlap S_W with a negative eigenvalue: LRES_ENUMERIC naming the window, on both routes;
* trace rows beyond the owned rows and a pass with mu <= e_lo: LRES_EINVAL;
* the context keeps working after each failure once clean matrices are set again."""
import ctypes as C

import numpy as np
import pytest

from golden_util import crystal, load

pytestmark = pytest.mark.gpu

BAD = 5          # the window that receives the fault


@pytest.fixture(scope="module")
def cubic3():
    from lresdft_gb300 import system
    g = load("cubic3")
    cr = crystal(g)
    return g, cr, system.LCAOBasis(cr)


def _solver(cubic3, precision, route):
    from lresdft_gb300 import LResGPU
    g, cr, b = cubic3
    s = LResGPU(b, cr.pos, R_w=float(g["R_w"]), M=int(g["M"]), precision=precision, route=route,
                trace_rows=False)
    s.set_potential(g["v"].reshape(cr.shape))
    return s


def _raw_pass(s, mu, e_lo):
    from lresdft_gb300 import _lib
    out = np.zeros(3)
    rc = _lib.lib.lres_pass(s._ctx, float(mu), float(e_lo), None, 0, _lib.ptrd(out), None)
    return rc, out, _lib.lib.lres_last_error().decode()


@pytest.mark.parametrize("route", ["tridiag", "ldl"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nan_in_one_window(cubic3, precision, route):
    from lresdft_gb300 import _lib
    g, cr, b = cubic3
    mu, e_lo = float(g["cold_mu"]), float(g["cold_elo"])
    s = _solver(cubic3, precision, route)
    from lresdft_gb300.autograd import window_matrices
    HW, SW = [t.cpu().numpy() for t in window_matrices(s)]
    rc, out, _ = _raw_pass(s, mu, e_lo)
    assert rc == 0 and out[2] == 0
    nw0, ew0 = s.window_sums()
    off = s.window_offsets
    n = int(s.ctx_nW[BAD])
    bad = HW.copy()
    blk = bad[off[BAD]:off[BAD + 1]].reshape(n, n, order="F")
    blk[3, 1] = blk[1, 3] = np.nan
    s.set_windows(HW=bad)
    rc, out, msg = _raw_pass(s, mu, e_lo)
    assert rc == -33
    assert int(out[2]) & 1, out
    assert "pivot" in msg
    nw, ew = s.window_sums()
    others = np.arange(len(nw)) != BAD
    assert not np.isfinite(nw[BAD]) or not np.isfinite(ew[BAD])
    assert np.array_equal(nw[others], nw0[others]) and np.array_equal(ew[others], ew0[others])
    with pytest.raises(_lib.NumericError):
        s.pole_pass(mu, e_lo)
    # clean matrices again: the context recovers
    s.set_windows(HW=HW)
    rc, out, _ = _raw_pass(s, mu, e_lo)
    assert rc == 0 and out[2] == 0
    nw1, ew1 = s.window_sums()
    assert np.array_equal(nw1, nw0) and np.array_equal(ew1, ew0)
    s.close()


@pytest.mark.parametrize("route", ["tridiag", "ldl"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_indefinite_overlap_is_reported(cubic3, precision, route):
    from lresdft_gb300 import _lib
    from lresdft_gb300.autograd import window_matrices
    g, cr, b = cubic3
    s = _solver(cubic3, precision, route)
    HW, SW = [t.cpu().numpy() for t in window_matrices(s)]
    off = s.window_offsets
    n = int(s.ctx_nW[BAD])
    bad = SW.copy()
    blk = bad[off[BAD]:off[BAD + 1]].reshape(n, n, order="F")
    lam, U = np.linalg.eigh(blk)
    blk[:] = blk - 2.0 * lam[-1] * np.outer(U[:, -1], U[:, -1])      # largest eigenvalue -> negative
    with pytest.raises(_lib.NumericError, match=f"window {BAD} is not positive definite"):
        s.set_windows(SW=bad)
    s.set_windows(HW=HW, SW=SW)
    d, N, E = s.pole_pass(float(g["cold_mu"]), float(g["cold_elo"]))
    assert abs(E - g["cold_eband"]) / cr.n_elec < 2e-7
    s.close()


def test_invalid_arguments_are_rejected(cubic3):
    from lresdft_gb300 import _lib
    g, cr, b = cubic3
    s = _solver(cubic3, "fp64", "tridiag")
    rc, out, msg = _raw_pass(s, -0.5, -0.2)                       # e_lo above mu
    assert rc == -22 and "e_lo < mu" in msg
    nwin = len(s.ctx_windows)
    r_w = np.full(nwin, 10 ** 6, np.int32)                        # more trace rows than owned rows
    R = np.zeros(8)
    rc = _lib.lib.lres_set_trace_rows(s._ctx, r_w.ctypes.data, R.ctypes.data, None)
    assert rc == -22 and b"trace rows" in _lib.lib.lres_last_error()
    rc = _lib.lib.lres_set_route(s._ctx, C.c_int32(7), None)
    assert rc == -22
    d, N, E = s.pole_pass(float(g["cold_mu"]), float(g["cold_elo"]))
    assert np.max(np.abs(d - g["cold_dens"])) < 1e-10
    s.close()
