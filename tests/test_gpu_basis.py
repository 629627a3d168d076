"""Basis tabulation on the GPU (lres_basis_tabulate) against the numpy tabulation, which
restates the reference's loop (lrft/lcao3d.py:61-84) operation by operation.

Gates: the same points (X has the same pattern, CSC and CSR), values within 1e-14 of the
largest basis value (CUDA's exp against numpy's: a few ulp; the normalisation sums in
another order), S and T within 1e-13 and 1e-11 in every entry of either pattern; the FP64
pole pass on the GPU-tabulated basis matches the reference's density to 1e-10."""
import numpy as np
import pytest

from golden_util import crystal, load

pytestmark = pytest.mark.gpu


def _dense_diff(A, B):
    D = (A - B).tocoo()
    return np.max(np.abs(D.data)) if D.nnz else 0.0


def _compare(bn, bg):
    assert bg.nb == bn.nb and np.array_equal(bg.atom_of_fn, bn.atom_of_fn)
    for A, B in ((bn.X, bg.X), (bn.Xr, bg.Xr)):
        assert np.array_equal(A.indptr, B.indptr) and np.array_equal(A.indices, B.indices)
    scale = np.max(np.abs(bn.X.data))
    assert np.max(np.abs(bg.X.data - bn.X.data)) <= 1e-14 * scale
    assert _dense_diff(bg.S, bn.S) < 1e-13
    assert _dense_diff(bg.T, bn.T) < 1e-11


@pytest.mark.parametrize("name", ["cubic3", "jit2"])
def test_gpu_tabulation_matches_numpy(name):
    from lresdft_gb300 import system
    g = load(name)
    cr = crystal(g)
    _compare(system.LCAOBasis(cr), system.LCAOBasis(cr, tabulation="gpu"))


def test_gpu_tabulation_per_atom_exponents():
    """Different exponent sets per atom (1, 4 and 8 functions), the 8x8x8 crystal's cell."""
    from lresdft_gb300 import system
    cr = system.jittered_h2((3, 3, 3), a=4.5, bond=1.4, pts_per_cell=8, jitter=0.1, seed=3)
    sets = [((1.0,), ()), ((1.0, 0.3), (0.5,)), ((1.0, 0.3), (0.5, 0.2))]
    atom_exps = [sets[a % 3] for a in range(len(cr.pos))]
    _compare(system.LCAOBasis(cr, atom_exps=atom_exps), system.LCAOBasis(cr, atom_exps=atom_exps, tabulation="gpu"))


def test_pass_on_gpu_tabulated_basis_matches_reference():
    from lresdft_gb300 import LResGPU, system
    g = load("cubic3")
    cr = crystal(g)
    b = system.LCAOBasis(cr, tabulation="gpu")
    s = LResGPU(b, cr.pos, R_w=float(g["R_w"]), M=int(g["M"]), precision="fp64")
    s.set_potential(g["v"].reshape(cr.shape))
    dens, N, eb = s.pole_pass(float(g["cold_mu"]), float(g["cold_elo"]))
    assert np.max(np.abs(dens - g["cold_dens"])) < 1e-10
    assert abs(eb - g["cold_eband"]) < 1e-9
    s.close()


def test_gpu_tabulation_1024_electrons():
    """The bench crystal (8x8x8 H2, 64^3 grid): same points and values as numpy."""
    from lresdft_gb300 import system
    cr = system.jittered_h2((8, 8, 8), a=4.5, bond=1.4, pts_per_cell=8, jitter=0.1, seed=0)
    _compare(system.LCAOBasis(cr), system.LCAOBasis(cr, tabulation="gpu"))
