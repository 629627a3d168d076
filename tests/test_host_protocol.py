"""The drop-in protocol of LResGPU (lresdft_gb300/solver.py: density(), the warm / cold mu
logic with the reference's edge test, lag_mu, trace-row passes) on the CPU.  A subclass
answers the solver's device calls (set_potential, pole_pass, inertia, min_eig) with the
oracle's eigen route on the host: window eigenpairs, r_M in closed form (lrft/lcao3d.py:
368-456, src/lrft_cpp.cpp:148-196), so the host logic runs unchanged over exact passes.

Pinned to the reference's three density calls (tests/golden/make_golden.py: cold call, warm
call with a forced mu re-solve, warm call that keeps mu) with the gates of the GPU protocol
test: 1e-9 in mu and E_band, 1e-10 in density."""
import numpy as np
import pytest

from golden_util import crystal, load


def _host_solver_class():
    from lresdft_gb300 import LResGPU
    from oracle import lrft_oracle as O

    class HostLRes(LResGPU):
        def __init__(self, basis, cells, R_w, M=64, margin=0.3, lag_mu=False, trace_rows=False):
            self.b, self.M, self.margin = basis, M, margin
            self.lag_mu, self.reuse_vectors, self.nthreads = lag_mu, False, 1
            self.precision = "fp64"
            self.windows, self.own, self.owner = O.window_setup(basis, np.asarray(cells, float), R_w)
            self.nW = np.array([len(W) for W in self.windows])
            self.ctx_windows, self._ctx_of = self.windows, np.arange(len(self.windows))
            self.mu = self.e_lo = None
            self.passes = self.inertia_calls = 0
            self._slope = self._mu_last = self._lam_min = None
            self.trace = None
            self._tuned, self.tile_config = True, None
            self._trace, self._resolved = bool(trace_rows), False
            self.trace_rows = None
            self._ctx = None

        def set_potential(self, v):
            b = self.b
            H = b.H(np.asarray(v, float).ravel())
            self._eig = []
            for W, o in zip(self.windows, self.own):
                lam, U = O.window_eig(H[W][:, W].toarray(), b.S[W][:, W].toarray(), np.inf)
                self._eig.append((lam, b.Xr[o][:, W] @ U, o))

        def pole_pass(self, mu, e_lo, want_density=True):
            self.passes += 1
            cr = self.b.cr
            dens = np.zeros(cr.ng) if want_density else None
            N = E = 0.0
            for lam, Y, o in self._eig:
                r = O.r_M(lam, mu, e_lo, self.M)
                c = np.sum(Y * Y, axis=0) * cr.dV
                N += 2.0 * np.dot(c, r)
                E += 2.0 * np.dot(c, lam * r)
                if want_density:
                    dens[o] = 2.0 * ((Y * Y) @ r)
            if self.trace is not None:
                self.trace.append((float(mu), N))
            return dens, N, E

        def inertia(self, sigma, per_window=False):
            self.inertia_calls += 1
            below = np.array([int(np.sum(lam < sigma)) for lam, _, _ in self._eig], np.int32)
            return below if per_window else int(below.sum())

        def min_eig(self, lo, hi, tol=1e-12):
            return float(min(lam.min() for lam, _, _ in self._eig))

    return HostLRes


@pytest.fixture(scope="module", params=["jit2", "cubic3"])
def case(request):
    from lresdft_gb300 import system
    g = load(request.param)
    cr = crystal(g)
    return g, cr, system.LCAOBasis(cr)


def _make(case, **kw):
    g, cr, b = case
    return _host_solver_class()(b, cr.pos, float(g["R_w"]), int(g["M"]), **kw)


def test_protocol_reproduces_reference_calls(case):
    g, cr, b = case
    s = _make(case)
    v = g["v"].reshape(cr.shape)
    n1, e1, mu1 = s.density(v)
    assert abs(s.e_lo - g["cold_elo"]) < 1e-9 and abs(mu1 - g["cold_mu"]) < 1e-9
    assert abs(e1 - g["cold_eband"]) < 1e-9 and np.max(np.abs(n1.ravel() - g["cold_dens"])) < 1e-10
    s.mu += 0.02
    n2, e2, mu2 = s.density(0.999 * v)
    assert abs(mu2 - g["warm_mu"]) < 1e-9 and abs(s.e_lo - g["warm_elo"]) < 1e-9
    assert abs(e2 - g["warm_eband"]) < 1e-9 and np.max(np.abs(n2.ravel() - g["warm_dens"])) < 1e-10
    p0 = s.passes
    n3, e3, mu3 = s.density(0.999 * v)
    assert s.passes - p0 == int(g["keep_passes"]) == 1 and mu3 == mu2
    assert abs(e3 - g["keep_eband"]) < 1e-9 and np.max(np.abs(n3.ravel() - g["keep_dens"])) < 1e-10


def test_trace_row_passes_give_the_same_calls(case):
    """With trace rows the trial passes return no density and the accepted mu gets one
    density pass: the same (density, E_band, mu) and the same trial points, plus one density
    pass per call (the cold call and the warm re-solve end on a trace-row pass; the call that
    keeps mu follows a re-solve, so its first pass runs over the trace rows too)."""
    g, cr, b = case
    v = g["v"].reshape(cr.shape)
    plain, traced = _make(case), _make(case, trace_rows=True)
    for s in (plain, traced):
        s.trace = []
    for step in range(3):
        if step == 1:
            plain.mu += 0.02
            traced.mu += 0.02
        vv = v if step == 0 else 0.999 * v
        a, b_ = plain.density(vv), traced.density(vv)
        assert abs(a[2] - b_[2]) < 1e-12 and abs(a[1] - b_[1]) < 1e-12
        assert np.max(np.abs(a[0] - b_[0])) < 1e-12
    assert traced.passes == plain.passes + 3
    it = iter(m for m, _ in traced.trace)
    assert all(any(m == t for t in it) for m, _ in plain.trace)     # plain's points, in order


def test_failed_edge_test_takes_the_cold_path(case):
    """A stale filter edge (lambda_min no longer within (e_lo + margin/3, e_lo + 2 margin),
    lrft/lcao3d.py:420) sends the next call down the cold path: a new e_lo and the cold
    call's result."""
    g, cr, b = case
    s = _make(case)
    v = g["v"].reshape(cr.shape)
    s.density(v)
    s.e_lo -= 1.0
    n, e, mu = s.density(v)
    assert abs(s.e_lo - g["cold_elo"]) < 1e-9 and abs(mu - g["cold_mu"]) < 1e-9
    assert abs(e - g["cold_eband"]) < 1e-9 and np.max(np.abs(n.ravel() - g["cold_dens"])) < 1e-10


def test_lag_mu_keeps_mu_for_a_small_count_error(case):
    """lag_mu=True: a warm call whose count is within 0.25 electrons keeps mu (one pass)."""
    g, cr, b = case
    s = _make(case, lag_mu=True)
    v = g["v"].reshape(cr.shape)
    _, _, mu1 = s.density(v)
    p0 = s.passes
    _, _, mu2 = s.density(0.9999 * v)
    assert mu2 == mu1 and s.passes - p0 == 1


def test_count_positive_at_the_bottom_raises(case):
    """The reference's RuntimeError when the count is positive at the bottom of the spectrum
    (lrft/lcao3d.py:391-392): here asked for a negative electron number."""
    g, cr, b = case
    s = _make(case)
    with pytest.raises(RuntimeError, match="bottom of the spectrum"):
        s.density(g["v"].reshape(cr.shape), N=-1.0)


def test_stale_mu_retries_cold(case):
    """StaleMu from a warm re-solve (no sign change of the count near the warm-start mu,
    lrft/lcao3d.py:400-405) makes density() drop mu and repeat the call cold."""
    from lresdft_gb300.solver import StaleMu
    g, cr, b = case
    s = _make(case)
    v = g["v"].reshape(cr.shape)
    s.density(v)
    solve = s._solve_mu
    raised = []

    def stale_once(e_lo, N, ftol, start=None, lo_start=None):
        if start is not None and not raised:
            raised.append(start[0])
            raise StaleMu("forced")
        return solve(e_lo, N, ftol, start=start, lo_start=lo_start)

    s._solve_mu = stale_once
    s.mu += 0.02
    n, e, mu = s.density(v)
    assert raised and abs(mu - g["cold_mu"]) < 1e-9 and abs(e - g["cold_eband"]) < 1e-9
    assert np.max(np.abs(n.ravel() - g["cold_dens"])) < 1e-10


def test_solve_mu_fixed_n(case):
    """solve_mu_fixed_n (the mu solve at fixed N behind BandEnergy and the finite-difference
    checks): a bracket grown from the current mu by slope steps, then Brent's method, to
    |N(mu) - N| <= tol on passes without density; the root of the closed-form count."""
    from scipy.optimize import brentq
    g, cr, b = case
    s = _make(case)
    v = g["v"].reshape(cr.shape)
    s.density(v)
    s.set_potential(1.002 * v)
    mu, N, E = s.solve_mu_fixed_n(tol=1e-10)
    assert abs(N - cr.n_elec) <= 1e-10

    def count(m):
        return s.pole_pass(m, s.e_lo, want_density=False)[1] - cr.n_elec
    ref = brentq(count, s.e_lo + 1e-6, s.mu + 1.0, xtol=1e-15)
    assert abs(mu - ref) < 1e-9
    assert abs(E - s.pole_pass(mu, s.e_lo, want_density=False)[2]) == 0.0


class _HostGrid:
    """The grid steps of the SCF driver answered by the oracle on the host."""

    def __init__(self, cr):
        self.cr = cr

    def ion_potential(self):
        from oracle import lrft_oracle as O
        return O.ion_potential(self.cr)

    def lda_hartree(self, dens):
        from oracle import lrft_oracle as O
        exc, vxc = O.lda_xc(dens)
        return exc, vxc, O.hartree(self.cr, dens)


def test_scf_driver_reproduces_reference_scf(case):
    """lresdft_gb300.scf.scf_lcao (DIIS over 6 histories, mix 0.4, clamp, renormalisation,
    Harris-Foulkes energy; lrft/lcao3d.py:237-284) over the host-backed solver and grid: the
    reference's LRFTLCAOCpp(reuse_vectors=False) SCF to tol 1e-8, same iteration count,
    energy to 1e-10 Ha/electron, final input density to 1e-9.  The pole passes the mu
    searches spend over the whole SCF stay within the counts of the current search (each one
    is a full GPU pass: 16 electrons 70 passes over 21 steps, 54 electrons 65 over 10)."""
    from lresdft_gb300.scf import scf_lcao
    g, cr, b = case
    s = _make(case)
    r = scf_lcao(cr, s, tol=1e-8, maxiter=60, grid=_HostGrid(cr))
    assert s.passes <= {16: 70, 54: 65}[cr.n_elec], s.passes
    assert r["converged"] and r["iterations"] == int(g["scf_iterations"])
    assert abs(r["energy"] - float(g["scf_energy"])) / cr.n_elec < 1e-10
    assert np.max(np.abs(r["dens_in"].ravel() - g["scf_dens_in"])) < 1e-9
