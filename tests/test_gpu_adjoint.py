"""Adjoint of the band energy at fixed N through the C ABI (lres_adjoint, lres_set_windows)
against the CPU oracle (oracle/lrft_adjoint.py: closed-form Daleckii-Krein derivative of
the eigen route, itself pinned to finite differences in tests/test_adjoint_oracle.py), against
central finite differences of the GPU forward (step 1e-5, 20 seeded directions each for the
grid potential, the window Hamiltonians and the window overlaps), and against the dense-KS
density-matrix gradient where every window is the whole cell.

Tolerances: FP64 path 1e-9 relative to the oracle, 1e-6 relative to finite differences
(norm over the 20 directions); mixed path 5e-5 relative to the oracle (measured worst case
1.5e-5, dN/dmu, on the 3x3x3 cell)."""
import numpy as np
import pytest

from golden_util import check_basis, crystal, load

pytestmark = pytest.mark.gpu

H_FD = 1e-5
NDIR = 20


@pytest.fixture(scope="module")
def cubic3():
    from lresdft_gb300 import system
    g = load("cubic3")
    cr = crystal(g)
    b = system.LCAOBasis(cr)
    check_basis(b, g)
    return g, cr, b


@pytest.fixture(scope="module")
def jit2():
    from lresdft_gb300 import system
    g = load("jit2")
    cr = crystal(g)
    b = system.LCAOBasis(cr)
    return g, cr, b


def _oracle(b, cr, s, v, mu, e_lo, M):
    """The oracle on the windows the GPU solves (``ctx_windows``: merged, atoms reordered), so
    that per-window gradients compare in the same layout."""
    from oracle.lrft_adjoint import adjoint
    return adjoint(b.H(v.ravel()), b.S, b.Xr, s.ctx_windows, s.ctx_own, cr.dV, mu, e_lo, M)


def _solver(b, cr, g, precision):
    from lresdft_gb300 import LResGPU
    return LResGPU(b, cr.pos, R_w=float(g["R_w"]), M=int(g["M"]), precision=precision)


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_adjoint_matches_oracle(cubic3, precision):
    g, cr, b = cubic3
    s = _solver(b, cr, g, precision)
    v = g["v"].reshape(cr.shape)
    mu, e_lo, M = float(g["cold_mu"]), float(g["cold_elo"]), int(g["M"])
    assert len(s.ctx_nW) == len(s.nW)           # no identical windows on this cell
    s.set_potential(v)
    a = s.adjoint(mu, e_lo, windows=True)
    o = _oracle(b, cr, s, v, mu, e_lo, M)
    tol = 1e-9 if precision == "fp64" else 5e-5
    errs = {"N": abs(a["N"] - o["N"]) / o["N"], "E": abs(a["E"] - o["E"]) / abs(o["E"]),
            "dNdmu": abs(a["dNdmu"] - o["dNdmu"]) / abs(o["dNdmu"]),
            "kappa": abs(a["kappa"] - o["kappa"]) / abs(o["kappa"]),
            "dv": _rel(a["dv"].ravel(), o["dv"]),
            "dHW": _rel(a["dHW"], s.flatten_windows(o["dH"])),
            "dSW": _rel(a["dSW"], s.flatten_windows(o["dS"]))}
    print(precision, {k: f"{x:.2e}" for k, x in errs.items()})
    for k, x in errs.items():
        assert x < tol, (k, x)
    s.close()


def _smooth_dirs(shape, n, seed):
    """Seeded smooth unit-RMS fields (a few random plane waves plus a little white noise)."""
    rng = np.random.default_rng(seed)
    I, J, K = np.meshgrid(*[np.arange(m) for m in shape], indexing="ij")
    out = []
    for _ in range(n):
        d = np.zeros(shape)
        for _ in range(4):
            kv = rng.integers(-2, 3, 3)
            ph = rng.uniform(0, 2 * np.pi)
            d += rng.normal() * np.cos(2 * np.pi * (kv[0] * I / shape[0] + kv[1] * J / shape[1] +
                                                    kv[2] * K / shape[2]) + ph)
        d += 0.3 * rng.normal(size=shape)
        out.append(d / np.sqrt(np.mean(d ** 2)))
    return out


def _sym_dirs(s, n, seed):
    """Seeded random symmetric window perturbations, unit Frobenius norm over all windows."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        mats = []
        for nw in s.ctx_nW:
            x = rng.normal(size=(nw, nw))
            mats.append(x + x.T)
        flat = s.flatten_windows(mats)
        out.append(flat / np.linalg.norm(flat))
    return out


def test_adjoint_matches_finite_differences_fp64(cubic3):
    """Central differences of E_band at fixed N (mu re-solved by secant passes to 1e-11
    electrons, first-order remainder removed with kappa) along 20 directions each."""
    g, cr, b = cubic3
    s = _solver(b, cr, g, "fp64")
    v = g["v"].reshape(cr.shape)
    N0 = float(cr.n_elec)
    s.density(v)
    mu0, e_lo = s.mu, s.e_lo
    mu0, _, _ = s.solve_mu_fixed_n(tol=1e-11)
    s.mu = mu0
    base = s.adjoint(mu0, e_lo, windows=True)
    kap = base["kappa"]
    from lresdft_gb300.autograd import window_matrices
    HW0, SW0 = [t.cpu().numpy() for t in window_matrices(s)]

    def energy():
        mu, N, E = s.solve_mu_fixed_n(mu0=mu0, tol=1e-11)
        return E - kap * (N - N0)

    results = {}
    for kind in ("v", "H", "S"):
        fd, an = [], []
        dirs = _smooth_dirs(cr.shape, NDIR, 11) if kind == "v" else _sym_dirs(s, NDIR, 12 if kind == "H" else 13)
        for d in dirs:
            e = []
            for sgn in (1, -1):
                if kind == "v":
                    s.set_potential(v + sgn * H_FD * d)
                elif kind == "H":
                    s.set_windows(HW=HW0 + sgn * H_FD * d)
                else:
                    s.set_windows(HW=HW0, SW=SW0 + sgn * H_FD * d)
                e.append(energy())
            fd.append((e[0] - e[1]) / (2 * H_FD))
            grad = {"v": base["dv"].ravel(), "H": base["dHW"], "S": base["dSW"]}[kind]
            an.append(float(np.dot(grad, d.ravel())))
        s.set_windows(HW=HW0, SW=SW0)
        fd, an = np.array(fd), np.array(an)
        results[kind] = float(np.linalg.norm(fd - an) / np.linalg.norm(an))
        print(kind, "rel err", results[kind], "max |an|", np.max(np.abs(an)))
    for kind, err in results.items():
        assert err < 1e-6, (kind, err)
    s.close()


def test_autograd_functions(cubic3):
    """BandEnergy / WindowBandEnergy backward equal the adjoint; forward is E at fixed N."""
    import torch
    from lresdft_gb300.autograd import BandEnergy, WindowBandEnergy, window_matrices
    g, cr, b = cubic3
    s = _solver(b, cr, g, "fp64")
    v = g["v"].reshape(cr.shape)
    s.density(v)
    vt = torch.tensor(v, dtype=torch.float64, device="cuda", requires_grad=True)
    E = BandEnergy.apply(vt, s)
    E.backward()
    ref = s.adjoint(s.mu, s.e_lo, windows=True)
    assert abs(float(E.detach()) - ref["E"]) < 1e-9 * abs(ref["E"])
    assert abs(ref["N"] - cr.n_elec) < 1e-9
    assert _rel(vt.grad.cpu().numpy().ravel(), ref["dv"].ravel()) < 1e-12
    HW, SW = window_matrices(s)
    HW.requires_grad_(True)
    SW.requires_grad_(True)
    E2 = WindowBandEnergy.apply(HW, SW, s)
    (2.0 * E2).backward()
    assert abs(float(E2.detach()) - float(E.detach())) < 1e-9 * abs(float(E.detach()))
    assert _rel(HW.grad.cpu().numpy(), 2.0 * ref["dHW"]) < 1e-9
    assert _rel(SW.grad.cpu().numpy(), 2.0 * ref["dSW"]) < 1e-9
    s.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_whole_cell_windows_equal_dense_ks_gradient(jit2, precision):
    """2x2x2 cell at R_w = 8: every window is the whole cell, so the sum of the window
    gradients is the dense-KS density-matrix gradient U diag(2r + 2(lam - kappa) r') U^T
    and dE/dv is its grid diagonal (LRes equals KS in this limit, tests/test_three_d.py:51-60)."""
    from oracle.lrft_adjoint import dense_ks_gradient
    g, cr, b = jit2
    s = _solver(b, cr, g, precision)
    assert all(n == b.nb for n in s.nW)
    v = g["v"].reshape(cr.shape)
    mu, e_lo = float(g["cold_mu"]), float(g["cold_elo"])
    s.set_potential(v)
    a = s.adjoint(mu, e_lo, windows=True)
    H = b.H(v.ravel())
    G, kap = dense_ks_gradient(H, b.S, cr.n_elec, cr.dV, mu, e_lo, int(g["M"]))
    gsum = sum(s.window_blocks(a["dHW"]))
    dv_ks = cr.dV * np.asarray(b.Xr.multiply(b.Xr @ G).sum(axis=1)).ravel()
    tol = 1e-9 if precision == "fp64" else 5e-5
    errs = (abs(a["kappa"] - kap) / abs(kap), _rel(gsum, G), _rel(a["dv"].ravel(), dv_ks))
    print(precision, errs)
    assert max(errs) < tol, errs
    s.close()
