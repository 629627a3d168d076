"""Trace rows (lres_owned_gram + lres_set_trace_rows): passes without a density and the
adjoint over R_W (R_W^T R_W = F_W^T F_W, at most n_W rows) instead of the owned grid points
give the same N(mu), E_band and gradients; the density call with trace rows (trial mu passes
over R_W, one density pass at the accepted mu) gives the same (density, E_band, mu).

Tolerances: FP64 1e-11 relative on N, E_band, 1e-10 on gradients and densities; mixed 1e-6."""
import numpy as np
import pytest

from golden_util import check_basis, crystal, load

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cubic3():
    from lresdft_gb300 import system
    g = load("cubic3")
    cr = crystal(g)
    b = system.LCAOBasis(cr)
    check_basis(b, g)
    return g, cr, b


def _solver(b, cr, R_w, M, precision, trace_rows):
    from lresdft_gb300 import LResGPU
    return LResGPU(b, cr.pos, R_w=R_w, M=M, precision=precision, trace_rows=trace_rows)


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_trace_rows_give_same_sums_and_gradient(cubic3, precision):
    g, cr, b = cubic3
    R_w, M = float(g["R_w"]), int(g["M"])
    mu, e_lo = float(g["cold_mu"]), float(g["cold_elo"])
    v = g["v"].reshape(cr.shape)
    full = _solver(b, cr, R_w, M, precision, False)
    tr = _solver(b, cr, R_w, M, precision, True)
    assert tr.trace_rows is not None and np.all(tr.trace_rows <= tr.ctx_nW)
    for s in (full, tr):
        s.set_potential(v)
    _, N0, E0 = full.pole_pass(mu, e_lo, want_density=False)
    _, N1, E1 = tr.pole_pass(mu, e_lo, want_density=False)
    a0 = full.adjoint(mu, e_lo, windows=True)
    a1 = tr.adjoint(mu, e_lo, windows=True)
    tol_s, tol_g = (1e-11, 1e-10) if precision == "fp64" else (1e-6, 1e-5)
    assert abs(N1 - N0) < tol_s * N0 and abs(E1 - E0) < tol_s * abs(E0)
    for k in ("dv", "dHW", "dSW"):
        assert _rel(np.ravel(a1[k]), np.ravel(a0[k])) < tol_g, k
    assert abs(a1["kappa"] - a0["kappa"]) < tol_g * abs(a0["kappa"])
    # a density pass still uses the owned points
    d0, _, _ = full.pole_pass(mu, e_lo)
    d1, _, _ = tr.pole_pass(mu, e_lo)
    assert _rel(d1, d0) < tol_g
    full.close()
    tr.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fine_grid_density_call_with_trace_rows(precision):
    """2x2x2 cell at 16 points per lattice constant (2048 owned points per 96-function
    window): trace rows are installed automatically and the density protocol returns what
    the owned-point passes return."""
    from lresdft_gb300 import system
    cr = system.jittered_h2((2, 2, 2), a=4.5, bond=1.4, pts_per_cell=16, jitter=0.1, seed=3)
    b = system.LCAOBasis(cr)
    from oracle.lrft_oracle import guess_potential
    v = guess_potential(cr)
    auto = _solver(b, cr, 8.0, 64, precision, "auto")
    assert auto.trace_rows is not None and auto.trace_rows.max() <= 96
    full = _solver(b, cr, 8.0, 64, precision, False)
    d1, e1, mu1 = auto.density(v)
    d0, e0, mu0 = full.density(v)
    tol = 1e-9 if precision == "fp64" else 1e-6
    assert abs(mu1 - mu0) < tol
    assert abs(e1 - e0) < tol * abs(e0)
    assert _rel(d1, d0) < tol * 10
    auto.close()
    full.close()
