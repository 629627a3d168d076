"""TEST INFRASTRUCTURE ONLY — the CPU oracle for the LRes-DFT LCAO window solve.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` import this module, and only as the checker or as the timed CPU
baseline; the product (``lresdft_gb300``) never calls it.

It restates, in numpy/scipy, the reference's algorithm for the path:

* window / Voronoi-ownership setup            lrft/lcao3d.py:132-161
* eigen route per window (dsygvd / dsygvx)    src/lrft_cpp.cpp:79-114,148-196; lrft/lcao3d.py:163-173
* closed-form occupation r_M                  lrft/three_d.py:221-225, src/lrft_cpp.cpp:69-74
* mu solve / warm-cold logic                  lrft/lcao3d.py:383-456 (LRFTLCAOCpp._density)
* pole nodes and weights                      lrft/core.py:130-139
* pole route on one window                    benchmarks/window_resolvent_vs_eig.py:35-36,58-65
* LDA, FFT Hartree, ion potential             lrft/three_d.py:90-148
* SCF driver (Pulay/DIIS, Harris-Foulkes)     lrft/lcao3d.py:237-284

The eigenvalue arithmetic is LAPACK's (scipy's bundled OpenBLAS), as in the
reference (build_cpp.sh links the system OpenBLAS).  Parity of this restatement
with the reference itself is pinned by ``tests/golden`` (vectors produced by
running the reference's own code, see tests/golden/make_golden.py) and by the
reference's published SCF energies (results/scaling_rigorous.json).
"""
from __future__ import annotations

import time

import numpy as np
import scipy.fft
from scipy import linalg
from scipy.optimize import brentq

from lresdft_gb300.system import Crystal, min_image


# --------------------------------------------------------------------------
# physics kernels (lrft/three_d.py)
# --------------------------------------------------------------------------

def gvectors(cr: Crystal):
    """lrft/three_d.py:90-92"""
    ks = [2 * np.pi * np.fft.fftfreq(m, d=L / m) for m, L in zip(cr.shape, cr.cell)]
    return np.meshgrid(*ks, indexing="ij")


def ion_potential(cr: Crystal):
    """Periodic sum of -Z erf(r/rc)/r through its structure factor (lrft/three_d.py:102-119)."""
    kx, ky, kz = gvectors(cr)
    G2 = kx**2 + ky**2 + kz**2
    vol = float(np.prod(cr.cell))
    S = np.zeros(cr.shape, complex)
    for (x, y, z), Z, rc in zip(cr.pos, cr.Z, cr.atom_rc):
        S += Z * np.exp(-1j * (kx * x + ky * y + kz * z) - G2 * rc**2 / 4)
    with np.errstate(divide="ignore", invalid="ignore"):
        vG = -4 * np.pi / G2 * S / vol
    vG[0, 0, 0] = 0.0
    return np.real(scipy.fft.ifftn(vG)) * cr.ng


def hartree(cr: Crystal, n):
    """v_H = IFFT(4 pi n(G) / G^2), G = 0 removed (lrft/three_d.py:122-129)."""
    kx, ky, kz = gvectors(cr)
    G2 = kx**2 + ky**2 + kz**2
    nG = scipy.fft.fftn(n)
    with np.errstate(divide="ignore", invalid="ignore"):
        vG = 4 * np.pi * nG / G2
    vG[0, 0, 0] = 0.0
    return np.real(scipy.fft.ifftn(vG))


def lda_xc(n):
    """Slater exchange + PZ81 correlation, unpolarised (lrft/three_d.py:132-148)."""
    n = np.maximum(n, 1e-14)
    rs = (3 / (4 * np.pi * n)) ** (1 / 3)
    ex = -0.75 * (3 / np.pi) ** (1 / 3) * n ** (1 / 3)
    vx = 4.0 / 3.0 * ex
    g, b1, b2 = -0.1423, 1.0529, 0.3334
    A, B, C, D = 0.0311, -0.048, 0.0020, -0.0116
    sr = np.sqrt(rs)
    den = 1 + b1 * sr + b2 * rs
    ec_hi = g / den
    vc_hi = ec_hi * (1 + 7 / 6 * b1 * sr + 4 / 3 * b2 * rs) / den
    lr = np.log(rs)
    ec_lo = A * lr + B + C * rs * lr + D * rs
    vc_lo = A * lr + (B - A / 3) + 2 / 3 * C * rs * lr + (2 * D - C) / 3 * rs
    hi = rs >= 1
    return ex + np.where(hi, ec_hi, ec_lo), vx + np.where(hi, vc_hi, vc_lo)


def r_M(lam, mu, e_lo, M):
    """Closed-form M-pole occupation 1/(1+u^M), u = (lam-c)/R (lrft/three_d.py:221-225)."""
    c, R = 0.5 * (mu + e_lo), 0.5 * (mu - e_lo)
    u = (lam - c) / R
    with np.errstate(over="ignore"):
        return 1.0 / (1.0 + u**M)


def nodes(M, mu, e_lo):
    """Upper-half-plane nodes z_j = c + R zeta_j and weights w_j = R zeta_j / M (lrft/core.py:130-139)."""
    assert M % 2 == 0
    c, R = 0.5 * (mu + e_lo), 0.5 * (mu - e_lo)
    zeta = np.exp(1j * np.pi * (2 * np.arange(M // 2) + 1) / M)
    return c + R * zeta, R * zeta / M


# --------------------------------------------------------------------------
# window / ownership setup (lrft/lcao3d.py:132-161)
# --------------------------------------------------------------------------

def window_setup(basis, cells, R_w):
    """Windows W(B) and Voronoi-owned grid points own(B), reference loop form."""
    cr = basis.cr
    d = min_image(cr.pos[:, None, :] - cells[None, :, :], cr.cell)
    cell_of_atom = np.argmin(np.linalg.norm(d, axis=2), axis=1)
    cell_of_fn = cell_of_atom[basis.atom_of_fn]
    dc = np.linalg.norm(min_image(cells[:, None, :] - cells[None, :, :], cr.cell), axis=2)
    I, J, K = np.meshgrid(*[np.arange(m) for m in cr.shape], indexing="ij")
    r = np.stack([I, J, K], -1).reshape(-1, 3) * cr.dx
    owner = np.empty(cr.ng, int)
    best = np.full(cr.ng, np.inf)
    for B, cB in enumerate(cells):
        dd = min_image(r - cB, cr.cell)
        d2 = np.einsum("ij,ij->i", dd, dd)
        m = d2 < best
        best[m] = d2[m]
        owner[m] = B
    windows, own = [], []
    for B in range(len(cells)):
        windows.append(np.where(np.isin(cell_of_fn, np.where(dc[B] <= R_w)[0]))[0])
        own.append(np.where(owner == B)[0])
    return windows, own, owner


# --------------------------------------------------------------------------
# eigen route (src/lrft_cpp.cpp:148-196, lrft/lcao3d.py:340-456)
# --------------------------------------------------------------------------

def window_eig(HW, SW, upper):
    """Generalised eigenpairs of one window: all (dsygvd) or those <= upper (dsygvx)."""
    if not np.isfinite(upper):
        return linalg.eigh(HW, SW, driver="gvd")
    return linalg.eigh(HW, SW, subset_by_value=(-np.inf, upper), driver="gvx")


def window_pass(H, S, Xr, windows, own, ng, dV, mu, e_lo, M, upper, want_density):
    """One pass over all windows, as _lrft_cpp.lrft_windows (src/lrft_cpp.cpp:129-233):
    returns (dens[ng] or None, lam, c, lamoff)."""
    dens = np.zeros(ng) if want_density else None
    lams, cs = [], []
    for W, o in zip(windows, own):
        HW, SW = H[W][:, W].toarray(), S[W][:, W].toarray()
        lam, U = window_eig(HW, SW, upper)
        Y = Xr[o][:, W] @ U
        c = np.sum(Y * Y, axis=0) * dV
        if want_density:
            dens[o] = (Y * Y) @ r_M(lam, mu, e_lo, M)
        lams.append(lam)
        cs.append(c)
    lamoff = np.concatenate([[0], np.cumsum([len(l) for l in lams])]).astype(np.int64)
    return dens, np.concatenate(lams), np.concatenate(cs), lamoff


class StaleMu(RuntimeError):
    """lrft/lcao3d.py:41-42"""


class LResEigenOracle:
    """Restatement of LRFTLCAOCpp with reuse_vectors=False (lrft/lcao3d.py:340-456):
    every mu re-solve is followed by a full second window pass, which is exactly
    what a pole-route solver does.  ``pool`` (optional) maps window passes over
    worker processes for large cases."""

    def __init__(self, basis, cells, R_w=12.1, M=64, margin=0.3, pool=None):
        self.b, self.M, self.margin = basis, M, margin
        self.windows, self.own, self.owner = window_setup(basis, cells, R_w)
        self.nW = np.array([len(W) for W in self.windows])
        self.mu = self.e_lo = None
        self.passes = 0
        self.pool = pool

    def _pass(self, H, mu, e_lo, upper, want_density):
        self.passes += 1
        b = self.b
        if self.pool is not None:
            return self.pool.window_pass(H, mu, e_lo, self.M, upper, want_density)
        return window_pass(H, b.S, b.Xr, self.windows, self.own, b.cr.ng, b.cr.dV, mu, e_lo, self.M,
                           upper, want_density)[:3]

    def _upper(self, mu, e_lo):
        c, R = 0.5 * (mu + e_lo), 0.5 * (mu - e_lo)
        return c + 1.5 * R

    def _solve_mu(self, lam, c, e_lo, N):
        def count(m):
            return 2.0 * np.dot(c, r_M(lam, m, e_lo, self.M)) - N
        lo = max(lam.min(), e_lo + 1e-6)
        if count(lo) > 0:
            raise RuntimeError("electron count positive at the bottom of the spectrum")
        hi = lo + 1.0
        while count(hi) < 0:
            hi += 0.5
            if hi > lam.max() + 10.0:
                raise StaleMu("truncated window spectra hold fewer than N electrons")
        return brentq(count, lo, hi, xtol=1e-12)

    def density(self, v, N=None, H=None):
        try:
            return self._density(v, N, H)
        except StaleMu:
            self.mu = None
            return self._density(v, N, H)

    def _density(self, v, N=None, H=None):
        b = self.b
        cr = b.cr
        N = cr.n_elec if N is None else N
        H = b.H(v) if H is None else H
        tol = 1e-8 * N
        if self.mu is not None:
            mu, e_lo = self.mu, self.e_lo
            dens, lam, c = self._pass(H, mu, e_lo, self._upper(mu, e_lo), True)
            if lam.size and e_lo + self.margin / 3 < lam.min() < e_lo + 2 * self.margin:
                cnt = 2.0 * np.dot(c, r_M(lam, mu, e_lo, self.M)) - N
                e_band = 2.0 * np.dot(c, lam * r_M(lam, mu, e_lo, self.M))
                if abs(cnt) > tol:
                    mu = self._solve_mu(lam, c, e_lo, N)
                    dens, lam, c = self._pass(H, mu, e_lo, self._upper(mu, e_lo), True)
                    e_band = 2.0 * np.dot(c, lam * r_M(lam, mu, e_lo, self.M))
                self.mu = mu
                return 2.0 * dens.reshape(cr.shape), e_band, mu
        _, lam, c = self._pass(H, 0.0, -1.0, np.inf, False)
        e_lo = lam.min() - self.margin
        mu = self._solve_mu(lam, c, e_lo, N)
        dens, lam, c = self._pass(H, mu, e_lo, self._upper(mu, e_lo), True)
        self.mu, self.e_lo = mu, e_lo
        e_band = 2.0 * np.dot(c, lam * r_M(lam, mu, e_lo, self.M))
        return 2.0 * dens.reshape(cr.shape), e_band, mu


# --------------------------------------------------------------------------
# pole route on one window (benchmarks/window_resolvent_vs_eig.py:35-36,58-65)
# --------------------------------------------------------------------------

def pole_window(HW, SW, F, mu, e_lo, M):
    """Owned-point density and band-energy density of one window by M/2 complex
    solves: d_k(r) = x_r^T (z_k S - H)^-1 x_r, n(r) = 2 sum_k 2 Re w_k d_k(r),
    e(r) = 2 sum_k 2 Re w_k z_k d_k(r).  F = X[own, W]^T (n x m).  Returns the
    spin-summed values (factor 2 of lrft/lcao3d.py:456 included)."""
    zs, ws = nodes(M, mu, e_lo)
    n = np.zeros(F.shape[1])
    e = np.zeros(F.shape[1])
    for z, w in zip(zs, ws):
        Y = linalg.solve(z * SW - HW, F.astype(complex))
        d = np.sum(F * Y, axis=0)
        n += 2 * np.real(w * d)
        e += 2 * np.real(w * z * d)
    return 2 * n, 2 * e


def pole_density(H, S, Xr, windows, own, ng, dV, mu, e_lo, M):
    """Pole-route density over all windows; returns (dens[ng], N, E_band)."""
    dens = np.zeros(ng)
    N = E = 0.0
    for W, o in zip(windows, own):
        HW, SW = H[W][:, W].toarray(), S[W][:, W].toarray()
        F = Xr[o][:, W].toarray().T
        nB, eB = pole_window(HW, SW, F, mu, e_lo, M)
        dens[o] = nB
        N += nB.sum() * dV
        E += eB.sum() * dV
    return dens, N, E


# --------------------------------------------------------------------------
# SCF driver (lrft/lcao3d.py:237-284)
# --------------------------------------------------------------------------

def scf_lcao(cr, solver, tol=1e-6, maxiter=60, mix=0.4, ndiis=6, verbose=False, dens0=None, vion=None):
    t0 = time.perf_counter()
    vion = ion_potential(cr) if vion is None else vion
    dens = np.full(cr.shape, cr.n_elec / (cr.ng * cr.dV)) if dens0 is None else dens0.copy()
    hist_n, hist_r = [], []
    converged = False
    for it in range(1, maxiter + 1):
        exc, vxc = lda_xc(dens)
        v = vion + hartree(cr, dens) + vxc
        out = solver.density(v)
        nout, eband = out[0], out[1]
        resid = nout - dens
        err = np.sum(np.abs(resid)) * cr.dV / cr.n_elec
        if verbose:
            print(f"  it {it:2d} |dn|/N = {err:.2e}", flush=True)
        if err < tol:
            converged = True
            break
        hist_n.append(dens.copy())
        hist_r.append(resid.copy())
        if len(hist_n) > ndiis:
            hist_n.pop(0)
            hist_r.pop(0)
        k = len(hist_n)
        if k > 1:
            Bm = np.empty((k + 1, k + 1))
            Bm[:k, :k] = [[np.vdot(ri, rj) for rj in hist_r] for ri in hist_r]
            Bm[k, :k] = Bm[:k, k] = 1.0
            Bm[k, k] = 0.0
            rhs = np.zeros(k + 1)
            rhs[k] = 1.0
            coef = np.linalg.lstsq(Bm, rhs, rcond=None)[0][:k]
            dens = sum(c * h for c, h in zip(coef, hist_n)) + mix * sum(c * r for c, r in zip(coef, hist_r))
        else:
            dens = dens + mix * resid
        dens = np.maximum(dens, 1e-12)
        dens *= cr.n_elec / (dens.sum() * cr.dV)
    vh = hartree(cr, dens)
    exc, vxc = lda_xc(dens)
    E_H = 0.5 * np.sum(dens * vh) * cr.dV
    E_xc = np.sum(dens * exc) * cr.dV
    E = eband - np.sum((vh + vxc) * dens) * cr.dV + E_H + E_xc
    return dict(energy=E, density=nout, iterations=it, time=time.perf_counter() - t0,
                converged=converged, dens_in=dens, eband=eband, E_H=E_H, E_xc=E_xc)


def guess_potential(cr, vion=None):
    """Potential of the uniform starting density (tests/test_three_d.py:13-15)."""
    d0 = np.full(cr.shape, cr.n_elec / (cr.ng * cr.dV))
    vion = ion_potential(cr) if vion is None else vion
    return vion + hartree(cr, d0) + lda_xc(d0)[1]
