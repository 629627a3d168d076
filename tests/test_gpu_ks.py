"""Dense Kohn-Sham LCAO on the GPU (lres_ks_density; ks_lcao, lrft/lcao3d.py:110-117) against
the same computation with scipy's generalised eigensolver (LAPACK dsygvx, as the reference's
ks_density, src/lrft_cpp.cpp:235-284), and the identity that the LRes density with one
whole-cell window equals it (the reference's test_three_d.py:18-35 check, run on the GPU).

Gates: eigenvalues 1e-10 Ha, band energy 1e-9 Ha, density 1e-10."""
import numpy as np
import pytest
from scipy import linalg

from golden_util import crystal, load

pytestmark = pytest.mark.gpu


def _scipy_ks(b, v):
    nocc = b.cr.n_elec // 2
    w, C = linalg.eigh(b.H(np.ravel(v)).toarray(), b.S.toarray(), subset_by_index=(0, nocc), driver="gvx")
    Y = b.Xr @ C[:, :nocc]
    return (2.0 * np.sum(Y * Y, axis=1)).reshape(b.cr.shape), 2.0 * w[:nocc].sum(), w


@pytest.mark.parametrize("name", ["cubic3", "jit2"])
def test_gpu_ks_matches_lapack(name):
    from lresdft_gb300 import ks, system
    g = load(name)
    cr = crystal(g)
    b = system.LCAOBasis(cr)
    v = g["v"].reshape(cr.shape)
    d0, e0, w0 = _scipy_ks(b, v)
    d1, e1, w1 = ks.ks_lcao(b, v)
    assert np.max(np.abs(w1 - w0)) < 1e-10
    assert abs(e1 - e0) < 1e-9
    assert np.max(np.abs(d1 - d0)) < 1e-10


def test_whole_cell_window_equals_gpu_ks():
    """One window holding every atom (R_w beyond the cell): the LRes density and band energy
    at a mu in the gap equal dense KS (the pole rule's error at M = 64 below the gates)."""
    from lresdft_gb300 import LResGPU, ks, system
    cr = system.h2_crystal((2, 2, 2), a=6.0, pts_per_cell=10, rc=0.6)
    b = system.LCAOBasis(cr, rcut=4.5, s_exps=(1.2, 0.4, 0.15), p_exps=(0.5,))
    from oracle import lrft_oracle as O
    v = O.guess_potential(cr)
    dk, ek, w = ks.ks_lcao(b, v)
    nocc = cr.n_elec // 2
    mu = 0.5 * (w[nocc - 1] + w[nocc])
    s = LResGPU(b, system.cell_centres((2, 2, 2), 6.0), R_w=100.0, M=64, precision="fp64")
    s.set_potential(v)
    lmin = s.min_eig(-5.0, 0.0, tol=1e-10)
    dens, N, eb = s.pole_pass(mu, lmin - 0.5)
    assert abs(N - cr.n_elec) < 1e-8
    assert abs(eb - ek) < 1e-8
    assert np.max(np.abs(dens - dk.ravel())) < 1e-8
    s.close()
