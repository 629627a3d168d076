"""The CPU oracle of the band-energy adjoint (oracle/lrft_adjoint.py) against central finite
differences of the reference's closed-form forward (eigen route, mu by brentq at fixed N),
step 1e-5 along 20 seeded directions each for the grid potential, the window Hamiltonians and
the window overlaps; and against the dense-KS density-matrix gradient when every window is
the whole cell.  2x2x2 H2 cell (16 electrons): R_w = 5 gives partial windows, R_w = 8 whole
ones."""
import numpy as np
import pytest

from golden_util import crystal, load

H_FD = 1e-5
NDIR = 20


@pytest.fixture(scope="module")
def sysjit2():
    from lresdft_gb300 import system
    g = load("jit2")
    cr = crystal(g)
    return g, cr, system.LCAOBasis(cr)


def _setup(b, cr, R_w):
    from oracle import lrft_oracle as O
    windows, own, _ = O.window_setup(b, cr.pos, R_w)
    return windows, own


def test_partial_windows(sysjit2):
    g, cr, b = sysjit2
    windows, own = _setup(b, cr, 5.0)
    nW = [len(W) for W in windows]
    assert min(nW) < b.nb
    assert max(nW) < b.nb


def test_oracle_adjoint_matches_finite_differences(sysjit2):
    from oracle.lrft_adjoint import adjoint, band_energy_fixed_N
    g, cr, b = sysjit2
    windows, own = _setup(b, cr, 5.0)
    M, dV, N0 = int(g["M"]), cr.dV, float(cr.n_elec)
    v = g["v"].ravel()
    H = b.H(v)
    e_lo = float(g["cold_elo"])
    HWs = [H[W][:, W].toarray() for W in windows]
    SWs = [b.S[W][:, W].toarray() for W in windows]
    Fs = [b.Xr[o][:, W].toarray().T for W, o in zip(windows, own)]
    _, mu0 = band_energy_fixed_N(HWs, SWs, Fs, dV, N0, e_lo, M, float(g["cold_mu"]))
    a = adjoint(H, b.S, b.Xr, windows, own, dV, mu0, e_lo, M)
    assert abs(a["N"] - N0) < 1e-10
    rng = np.random.default_rng(2024)
    I, J, K = np.meshgrid(*[np.arange(m) for m in cr.shape], indexing="ij")
    errs = {}
    for kind in ("v", "H", "S"):
        fd, an = [], []
        for _ in range(NDIR):
            if kind == "v":
                d = np.zeros(cr.shape)
                for _ in range(4):
                    kv = rng.integers(-2, 3, 3)
                    d += rng.normal() * np.cos(2 * np.pi * (kv[0] * I + kv[1] * J + kv[2] * K) / cr.shape[0]
                                               + rng.uniform(0, 2 * np.pi))
                d += 0.3 * rng.normal(size=cr.shape)
                d = (d / np.sqrt(np.mean(d ** 2))).ravel()
                e = [band_energy_fixed_N([b.H(v + sg * H_FD * d)[W][:, W].toarray() for W in windows], SWs, Fs,
                                         dV, N0, e_lo, M, mu0)[0] for sg in (1, -1)]
                an.append(np.dot(a["dv"], d))
            else:
                ds = [rng.normal(size=(len(W), len(W))) for W in windows]
                ds = [x + x.T for x in ds]
                nrm = np.sqrt(sum((x ** 2).sum() for x in ds))
                ds = [x / nrm for x in ds]
                if kind == "H":
                    e = [band_energy_fixed_N([A + sg * H_FD * x for A, x in zip(HWs, ds)], SWs, Fs, dV, N0, e_lo,
                                             M, mu0)[0] for sg in (1, -1)]
                    an.append(sum((gg * x).sum() for gg, x in zip(a["dH"], ds)))
                else:
                    e = [band_energy_fixed_N(HWs, [A + sg * H_FD * x for A, x in zip(SWs, ds)], Fs, dV, N0, e_lo,
                                             M, mu0)[0] for sg in (1, -1)]
                    an.append(sum((gg * x).sum() for gg, x in zip(a["dS"], ds)))
            fd.append((e[0] - e[1]) / (2 * H_FD))
        fd, an = np.array(fd), np.array(an)
        errs[kind] = float(np.linalg.norm(fd - an) / np.linalg.norm(an))
    assert max(errs.values()) < 1e-6, errs


def test_oracle_whole_cell_equals_dense_ks(sysjit2):
    from oracle.lrft_adjoint import adjoint, dense_ks_gradient
    g, cr, b = sysjit2
    windows, own = _setup(b, cr, 8.0)
    assert all(len(W) == b.nb for W in windows)
    M, mu, e_lo = int(g["M"]), float(g["cold_mu"]), float(g["cold_elo"])
    H = b.H(g["v"].ravel())
    a = adjoint(H, b.S, b.Xr, windows, own, cr.dV, mu, e_lo, M)
    G, kap = dense_ks_gradient(H, b.S, cr.n_elec, cr.dV, mu, e_lo, M)
    assert abs(a["kappa"] - kap) < 1e-12 * abs(kap)
    assert np.max(np.abs(a["gH"] - G)) < 1e-12 * np.max(np.abs(G))


def test_pole_route_mu_derivatives_and_gradients(sysjit2):
    """The combination lres_adjoint evaluates (lresdft_gb300/csrc/adjoint.cu), restated on the
    pole route in numpy: A_c = Re sum_k c_k Z_k Z_k^T with Z_k = (z_k S - H)^-1 F^T and c in
    {w, wz, wz^2}, U_c = 4 dV <S, A_c>; with a0 = 1/2 - c/(2R), a1 = 1/(2R):
        dN/dmu = N/(2R) - (a0 U_w + a1 U_wz),
        dE/dmu = E/R + N/2 - c N/(2R) - (a0 U_wz + a1 U_wz2),
        dE/dH_W = 4 dV (A_wz - kappa A_w),  dE/dS_W = -4 dV (A_wz2 - kappa A_wz),
    against the oracle's closed-form (eigen-route) derivatives."""
    from scipy import linalg
    from oracle import lrft_oracle as O
    from oracle.lrft_adjoint import adjoint
    g, cr, b = sysjit2
    windows, own = _setup(b, cr, 5.0)
    M, dV = int(g["M"]), cr.dV
    mu, e_lo = float(g["cold_mu"]), float(g["cold_elo"])
    H = b.H(g["v"].ravel())
    zs, ws = O.nodes(M, mu, e_lo)
    N = E = 0.0
    U = np.zeros(3)
    As = []
    for W, o in zip(windows, own):
        HW, SW = H[W][:, W].toarray(), b.S[W][:, W].toarray()
        F = b.Xr[o][:, W].toarray()                       # m x n
        A = np.zeros((3, len(W), len(W)))
        for z, w in zip(zs, ws):
            Z = linalg.solve(z * SW - HW, F.T.astype(complex))
            t = np.sum(F.T * Z)                          # tr(G F^T F)
            N += 4 * dV * np.real(w * t)
            E += 4 * dV * np.real(w * z * t)
            P = Z @ Z.T
            for c, cw in enumerate((w, w * z, w * z * z)):
                A[c] += np.real(cw * P)
        As.append(A)
        for c in range(3):
            U[c] += 4 * dV * np.sum(SW * A[c])
    cc, R = 0.5 * (mu + e_lo), 0.5 * (mu - e_lo)
    a0, a1 = 0.5 - cc / (2 * R), 1 / (2 * R)
    dN = N / (2 * R) - (a0 * U[0] + a1 * U[1])
    dE = E / R + 0.5 * N - cc * N / (2 * R) - (a0 * U[1] + a1 * U[2])
    kappa = dE / dN
    o = adjoint(H, b.S, b.Xr, windows, own, dV, mu, e_lo, M)
    assert abs(N - o["N"]) < 1e-10 * o["N"] and abs(E - o["E"]) < 1e-10 * abs(o["E"])
    assert abs(dN - o["dNdmu"]) < 1e-9 * abs(o["dNdmu"])
    assert abs(dE - o["dEdmu"]) < 1e-9 * abs(o["dEdmu"])
    for A, gH, gS in zip(As, o["dH"], o["dS"]):
        assert np.max(np.abs(4 * dV * (A[1] - kappa * A[0]) - gH)) < 1e-9 * np.max(np.abs(gH))
        assert np.max(np.abs(-4 * dV * (A[2] - kappa * A[1]) - gS)) < 1e-9 * np.max(np.abs(gS))
