"""The CPU oracle and the host-side system setup, pinned against vectors produced by
the reference's own code (tests/golden/make_golden.py) and against the reference's
published SCF energy (results/scaling_rigorous.json)."""
import numpy as np
import pytest

from golden_util import check_basis, crystal, load
from lresdft_gb300 import system
from oracle import lrft_oracle as orc


@pytest.fixture(scope="module", params=["jit2", "cubic3"])
def case(request):
    g = load(request.param)
    cr = crystal(g)
    b = system.LCAOBasis(cr)
    return request.param, g, cr, b


def test_generators_match_fixture_geometry():
    assert np.array_equal(system.h2_crystal((2, 2, 2)).pos, load("jit2")["pos"])
    assert np.array_equal(system.cubic_h2((3, 3, 3)).pos, load("cubic3")["pos"])


def test_basis_matches_reference(case):
    _, g, cr, b = case
    check_basis(b, g)


def test_potential_kernels_match_reference(case):
    _, g, cr, b = case
    vion = orc.ion_potential(cr)
    assert np.max(np.abs(vion.ravel() - g["vion"])) < 1e-12
    v = orc.guess_potential(cr, vion)
    assert np.max(np.abs(v.ravel() - g["v"])) < 1e-12


def test_window_setup_matches_reference(case):
    _, g, cr, b = case
    W, own, owner = orc.window_setup(b, cr.pos, float(g["R_w"]))
    assert np.array_equal(owner, g["owner"])
    assert np.array_equal(np.concatenate(W), g["Wflat"])
    assert np.array_equal([len(w) for w in W], g["nW"])


def test_eigen_oracle_reproduces_reference_density_calls(case):
    _, g, cr, b = case
    v = g["v"].reshape(cr.shape)
    o = orc.LResEigenOracle(b, cr.pos, R_w=float(g["R_w"]), M=int(g["M"]))
    n1, e1, mu1 = o.density(v)
    assert abs(e1 - g["cold_eband"]) < 1e-10 and abs(mu1 - g["cold_mu"]) < 1e-10
    assert np.max(np.abs(n1.ravel() - g["cold_dens"])) < 1e-11
    assert abs(o.e_lo - g["cold_elo"]) < 1e-12
    o.mu += 0.02
    n2, e2, mu2 = o.density(0.999 * v)
    assert abs(e2 - g["warm_eband"]) < 1e-10 and abs(mu2 - g["warm_mu"]) < 1e-10
    assert np.max(np.abs(n2.ravel() - g["warm_dens"])) < 1e-11
    p0 = o.passes
    n3, e3, mu3 = o.density(0.999 * v)
    assert o.passes - p0 == int(g["keep_passes"]) == 1
    assert abs(e3 - g["keep_eband"]) < 1e-10 and mu3 == pytest.approx(float(g["keep_mu"]), abs=1e-12)


def test_pole_route_equals_eigen_route(case):
    """Lemma 1 on every window: 2 Re sum_k w_k x^T (z_k S - H)^-1 x equals the closed-form
    r_M occupation of the window spectrum (tests/test_lrft.py:42-56 pins it to 1e-12)."""
    _, g, cr, b = case
    v = g["v"].reshape(cr.shape)
    W, own, _ = orc.window_setup(b, cr.pos, float(g["R_w"]))
    dens, N, E = orc.pole_density(b.H(v), b.S, b.Xr, W, own, cr.ng, cr.dV,
                                  float(g["cold_mu"]), float(g["cold_elo"]), int(g["M"]))
    assert np.max(np.abs(dens - g["cold_dens"])) < 1e-11
    assert abs(E - g["cold_eband"]) < 1e-10
    assert abs(N - cr.n_elec) < 1e-7


@pytest.mark.slow
def test_eigen_oracle_scf_matches_reference(case):
    name, g, cr, b = case
    o = orc.LResEigenOracle(b, cr.pos, R_w=float(g["R_w"]), M=int(g["M"]))
    r = orc.scf_lcao(cr, o, tol=1e-8)
    assert r["converged"] and r["iterations"] == int(g["scf_iterations"])
    assert abs(r["energy"] - g["scf_energy"]) / cr.n_elec < 1e-11


@pytest.mark.slow
def test_eigen_oracle_reproduces_published_energy():
    """results/scaling_rigorous.json, n=3: E_LRes(54 e) = -15.746532895084757 (a=6, 10 points
    per cell, rc=0.6, benchmark basis, cell windows R_w=12.1, M=64, tol 1e-6).  The published
    run used reuse_vectors=True (float32 |phi|^2), which moves the energy by ~1e-9."""
    cr = system.h2_crystal((3, 3, 3), a=6.0, pts_per_cell=10, rc=0.6)
    b = system.LCAOBasis(cr, rcut=4.5, s_exps=(1.2, 0.4, 0.15), p_exps=(0.5,))
    o = orc.LResEigenOracle(b, system.cell_centres((3, 3, 3), 6.0), R_w=12.1, M=64)
    r = orc.scf_lcao(cr, o, tol=1e-6)
    assert r["converged"] and r["iterations"] == 11
    assert abs(r["energy"] - (-15.746532895084757)) < 5e-9
