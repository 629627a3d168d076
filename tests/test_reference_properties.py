"""The reference's physics checks of this path (its tests/test_three_d.py:18-83), restated on
the CPU for this build.  Covered: the oracle's LDA and ion potential, and the solver protocol
of LResGPU over oracle-backed passes (see tests/test_host_protocol.py).  The protocol is
compared against dense LCAO Kohn-Sham on the same Hamiltonian: whole-cell windows equal KS,
the window error decays with R_w, and the LRes SCF reaches the KS SCF energy.  Same systems
and gates as the reference: a = 6 bohr, 10 points per cell, rc = 0.6, the benchmark basis."""
import numpy as np
import pytest
from scipy import linalg

from test_host_protocol import _HostGrid, _host_solver_class

BASIS = dict(rcut=4.5, s_exps=(1.2, 0.4, 0.15), p_exps=(0.5,))


def _system(n):
    from lresdft_gb300 import system
    cr = system.h2_crystal(n, a=6.0, pts_per_cell=10, rc=0.6)
    return cr, system.LCAOBasis(cr, **BASIS)


def _guess_v(cr):
    from oracle import lrft_oracle as O
    return O.guess_potential(cr)


def _ks_lcao(b, v):
    """Dense LCAO Kohn-Sham (lrft/lcao3d.py:110-117): the lowest N/2 generalised eigenpairs
    doubly occupied; returns (density, band energy)."""
    nocc = b.cr.n_elec // 2
    w, C = linalg.eigh(b.H(np.ravel(v)).toarray(), b.S.toarray(), subset_by_index=(0, nocc), driver="gvx")
    Y = b.Xr @ C[:, :nocc]
    return (2.0 * np.sum(Y * Y, axis=1)).reshape(b.cr.shape), 2.0 * w[:nocc].sum()


class _KS:
    def __init__(self, b):
        self.b = b

    def density(self, v):
        n, e = _ks_lcao(self.b, v)
        return n, e, None


def test_lda_potential_is_derivative():
    from oracle.lrft_oracle import lda_xc
    n = np.logspace(-4, 1, 40)
    e, v = lda_xc(n)
    h = 1e-6 * n
    fd = ((n + h) * lda_xc(n + h)[0] - (n - h) * lda_xc(n - h)[0]) / (2 * h)
    assert np.max(np.abs(fd - v) / np.abs(v)) < 1e-6


def test_ion_potential_is_neutral_and_attractive():
    from lresdft_gb300 import system
    from oracle.lrft_oracle import ion_potential
    cr = system.h2_crystal((1, 1, 1), a=6.0, pts_per_cell=10, rc=0.6)
    v = ion_potential(cr)
    assert abs(v.mean()) < 1e-10
    r = np.array(np.unravel_index(np.argmin(v), v.shape)) * cr.dx
    assert min(np.linalg.norm(r - p) for p in cr.pos) < 1.0


def test_whole_cell_windows_equal_ks():
    """R_w covering the periodic cell: every window is the whole basis and LRes equals KS up
    to the e^-M filter tail (E_band 1e-10 Ha, integrated |dn| 1e-9)."""
    from lresdft_gb300 import system
    n = (2, 2, 2)
    cr, b = _system(n)
    v = _guess_v(cr)
    nk, ek = _ks_lcao(b, v)
    s = _host_solver_class()(b, system.cell_centres(n, 6.0), 20.0, 64)
    assert all(len(W) == b.nb for W in s.windows)
    nl, el, _ = s.density(v)
    assert abs(el - ek) < 1e-10
    assert np.sum(np.abs(nl - nk)) * cr.dV < 1e-9


def test_window_error_decays():
    """4x4x4 cells: the density error against KS falls by 100x from R_w = 6.1 to 12.1 and ends
    below 1e-5 per electron."""
    from lresdft_gb300 import system
    n = (4, 4, 4)
    cr, b = _system(n)
    v = _guess_v(cr)
    nk, _ = _ks_lcao(b, v)
    errs = []
    for R_w in (6.1, 12.1):
        nl, _, _ = _host_solver_class()(b, system.cell_centres(n, 6.0), R_w, 64).density(v)
        errs.append(np.sum(np.abs(nl - nk)) * cr.dV / cr.n_elec)
    assert errs[1] < 1e-2 * errs[0] and errs[1] < 1e-5, errs


def test_scf_matches_ks():
    """LRes SCF (R_w = 12.1, cell windows) and KS SCF with the same driver to tol 1e-8: energies
    within 1e-8 Ha per electron."""
    from lresdft_gb300 import system
    from lresdft_gb300.scf import scf_lcao
    n = (2, 2, 2)
    cr, b = _system(n)
    ks = scf_lcao(cr, _KS(b), tol=1e-8, grid=_HostGrid(cr))
    lr = scf_lcao(cr, _host_solver_class()(b, system.cell_centres(n, 6.0), 12.1, 64), tol=1e-8, grid=_HostGrid(cr))
    assert ks["converged"] and lr["converged"]
    assert abs(lr["energy"] - ks["energy"]) / cr.n_elec < 1e-8
