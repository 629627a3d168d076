"""TEST INFRASTRUCTURE ONLY — CPU oracle of the band-energy adjoint of the LRes window solve.

The reference has no gradient code; its forward quantities are restated in
``oracle/lrft_oracle.py`` (eigen route, lrft/lcao3d.py:340-456 and src/lrft_cpp.cpp:148-196):

    N      = sum_B sum_i 2 c_i r_M(lam_i)            (lrft/lcao3d.py:389)
    E_band = sum_B sum_i 2 c_i lam_i r_M(lam_i)      (lrft/lcao3d.py:455)

with (lam_i, u_i) the S_W-orthonormal eigenpairs of window B and c_i = u_i^T O_B u_i,
O_B = dV X[own(B), W]^T X[own(B), W].  The reference's only derivative check is the
finite-M Hellmann-Feynman test tests/test_lrft.py:59-79; this module differentiates the
same closed form exactly:

* For E = tr(f(H_W, S_W) O_B) with f = U diag(phi(lam)) U^T the derivative is the
  Daleckii-Krein form dE/dH_W = U (Gamma_phi o U^T O_B U) U^T, Gamma_phi the matrix of
  divided differences of phi; the pole rule gives dE/dS_W = -U (Gamma_{lam phi} o ...) U^T
  (the node sum of w_k z_k^2 / (z_k - lam) equals 2 lam^2 r_M because sum_k w_k z_k = 0).
* At fixed N the chemical potential moves: dE|_N = dE - kappa dN with
  kappa = (dE/dmu) / (dN/dmu), e_lo held fixed (lrft/lcao3d.py:451 sets it once per
  cold start).
* The local potential enters through H = T + X^T diag(v) X dV (lrft/lcao3d.py:98-100):
  dE/dv(r) = dV sum_B x_{r,W}^T (dE/dH_W) x_{r,W}.

``band_energy_fixed_N`` is the matching forward (mu by brentq to 1e-15) used for central
finite differences; ``dense_ks_gradient`` is the dense Kohn-Sham density-matrix gradient that
the window gradient must equal when every window is the whole cell (S = X^T X dV, so
U^T S U = I and only the diagonal of Gamma survives).
"""
from __future__ import annotations

import numpy as np
from scipy import linalg
from scipy.optimize import brentq

from oracle.lrft_oracle import r_M


def dr_dmu(lam, mu, e_lo, M):
    """d r_M / d mu at fixed e_lo: M r (1 - r) (1 + u) / (2 R u), u = (lam - c)/R."""
    c, R = 0.5 * (mu + e_lo), 0.5 * (mu - e_lo)
    u = (lam - c) / R
    r = r_M(lam, mu, e_lo, M)
    with np.errstate(divide="ignore", invalid="ignore"):
        out = M * r * (1.0 - r) * (1.0 + u) / (2.0 * R * u)
    return np.where(np.abs(u) < 1e-300, 0.0, out)


def dr_dlam(lam, mu, e_lo, M):
    """d r_M / d lam = -M r (1 - r) / (R u)."""
    c, R = 0.5 * (mu + e_lo), 0.5 * (mu - e_lo)
    u = (lam - c) / R
    r = r_M(lam, mu, e_lo, M)
    with np.errstate(divide="ignore", invalid="ignore"):
        out = -M * r * (1.0 - r) / (R * u)
    return np.where(np.abs(u) < 1e-300, 0.0, out)


def _divided(phi, dphi, lam):
    """Gamma_ij = (phi_i - phi_j)/(lam_i - lam_j), phi'(lam_i) where lam_i == lam_j (to 1e-9)."""
    d = lam[:, None] - lam[None, :]
    close = np.abs(d) <= 1e-9 * max(1.0, np.max(np.abs(lam)))
    with np.errstate(divide="ignore", invalid="ignore"):
        G = (phi[:, None] - phi[None, :]) / d
    avg = 0.5 * (dphi[:, None] + dphi[None, :])
    return np.where(close, avg, G)


def window_parts(HW, SW, F, dV, mu, e_lo, M):
    """Per-window pieces of the adjoint: (N_B, E_B, dN/dmu_B, dE/dmu_B, and the four
    partial gradients dN/dH, dE/dH, dN/dS, dE/dS at fixed mu).  F = X[own, W]^T (n x m)."""
    lam, U = linalg.eigh(HW, SW, driver="gvd")
    Y = F.T @ U
    O = dV * (Y.T @ Y)                                   # U^T O_B U
    c = np.diag(O).copy()
    r = r_M(lam, mu, e_lo, M)
    rp = dr_dlam(lam, mu, e_lo, M)
    rm = dr_dmu(lam, mu, e_lo, M)
    N = 2 * np.dot(c, r)
    E = 2 * np.dot(c, lam * r)
    dNdmu = 2 * np.dot(c, rm)
    dEdmu = 2 * np.dot(c, lam * rm)
    f0, d0 = 2 * r, 2 * rp                               # N:  2 r
    f1, d1 = 2 * lam * r, 2 * (r + lam * rp)             # E:  2 lam r   (also -dN/dS)
    f2, d2 = 2 * lam**2 * r, 2 * (2 * lam * r + lam**2 * rp)   # -dE/dS: 2 lam^2 r
    parts = {}
    for name, (f, df, sgn) in {"NH": (f0, d0, 1), "EH": (f1, d1, 1), "NS": (f1, d1, -1),
                               "ES": (f2, d2, -1)}.items():
        parts[name] = sgn * (U @ (_divided(f, df, lam) * O) @ U.T)
    return N, E, dNdmu, dEdmu, parts


def adjoint(H, S, Xr, windows, own, dV, mu, e_lo, M):
    """Band-energy gradient at fixed N.  Returns dict with N, E, dN/dmu, dE/dmu, kappa,
    dH (list of per-window dE/dH_W), dS (list of dE/dS_W), gH (global nb x nb dense
    sum of the window gradients) and dv (dE/dv on the grid)."""
    res = [window_parts(H[W][:, W].toarray(), S[W][:, W].toarray(), Xr[o][:, W].toarray().T, dV, mu, e_lo, M)
           for W, o in zip(windows, own)]
    N = sum(r[0] for r in res)
    E = sum(r[1] for r in res)
    dNdmu = sum(r[2] for r in res)
    dEdmu = sum(r[3] for r in res)
    kappa = dEdmu / dNdmu
    dH = [p["EH"] - kappa * p["NH"] for *_, p in res]
    dS = [p["ES"] - kappa * p["NS"] for *_, p in res]
    nb = H.shape[0]
    gH = np.zeros((nb, nb))
    for W, g in zip(windows, dH):
        gH[np.ix_(W, W)] += g
    XG = Xr @ gH
    dv = dV * np.asarray(Xr.multiply(XG).sum(axis=1)).ravel()
    return {"N": N, "E": E, "dNdmu": dNdmu, "dEdmu": dEdmu, "kappa": kappa, "dH": dH, "dS": dS,
            "gH": gH, "dv": dv}


def _count_energy(lam_c, mu, e_lo, M):
    lam, c = lam_c
    r = r_M(lam, mu, e_lo, M)
    return 2 * np.dot(c, r), 2 * np.dot(c, lam * r)


def window_spectra(HWs, SWs, Fs, dV):
    """(lam, c) of all windows (full spectra) for the closed-form count and energy."""
    lams, cs = [], []
    for HW, SW, F in zip(HWs, SWs, Fs):
        lam, U = linalg.eigh(HW, SW, driver="gvd")
        Y = F.T @ U
        lams.append(lam)
        cs.append(dV * np.sum(Y * Y, axis=0))
    return np.concatenate(lams), np.concatenate(cs)


def band_energy_fixed_N(HWs, SWs, Fs, dV, N, e_lo, M, mu_guess):
    """E_band at fixed N with e_lo fixed: mu by brentq (xtol 1e-15) on the closed-form count."""
    lc = window_spectra(HWs, SWs, Fs, dV)

    def f(m):
        return _count_energy(lc, m, e_lo, M)[0] - N
    lo, hi = mu_guess - 0.05, mu_guess + 0.05
    while f(lo) > 0:
        lo -= 0.05
    while f(hi) < 0:
        hi += 0.05
    mu = brentq(f, lo, hi, xtol=1e-15, rtol=4 * np.finfo(float).eps, maxiter=500)
    return _count_energy(lc, mu, e_lo, M)[1], mu


def dense_ks_gradient(H, S, N, dV_unused, mu, e_lo, M):
    """Dense-KS density-matrix gradient of E_band = sum_i 2 lam_i r_M(lam_i) at fixed N:
    dE/dH = U diag(2 r + 2 (lam - kappa) r') U^T with kappa from the mu derivatives,
    the limit of the window gradient when every window is the whole cell."""
    lam, U = linalg.eigh(H.toarray(), S.toarray(), driver="gvd")
    r = r_M(lam, mu, e_lo, M)
    rp = dr_dlam(lam, mu, e_lo, M)
    rm = dr_dmu(lam, mu, e_lo, M)
    kappa = np.dot(lam, rm) / np.sum(rm)
    g = 2 * r + 2 * (lam - kappa) * rp
    return (U * g) @ U.T, kappa
