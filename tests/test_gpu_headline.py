"""The 1024-electron workload of the benchmark (8x8x8 H2, a = 4.5 bohr, centres jittered by
U(+-0.1) bohr, random bond axes, seed 0, 64^3 grid, one window per atom, R_w = 8 bohr, M = 64)
against the reference's own density call on it (tests/golden/jit8.npz, produced by the
reference's LRFTLCAOCpp: the potential of the uniform starting density, the cold call's mu and
e_lo, the band energy and 8192 sampled grid densities).

Gates: FP64 1e-10 on the sampled densities and 1e-9 Ha on the band energy (the reference's own
C++-vs-Python gate, tests/test_three_d.py:86-100); mixed precision 2e-7 Ha/electron on the band
energy and 1e-6 on the densities.  Both routes of the FP64 path are checked (the LDL^T route
costs seconds per pass at this size)."""
import numpy as np
import pytest

from golden_util import load

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def jit8():
    from lresdft_gb300 import LResGPU, system
    from lresdft_gb300.scf import GridOps
    g = load("jit8")
    cr = system.jittered_h2((8, 8, 8), a=4.5, bond=1.4, pts_per_cell=8, jitter=0.1, seed=0)
    b = system.LCAOBasis(cr)
    s = LResGPU(b, cr.pos, R_w=8.0, M=64, precision="fp64")
    go = GridOps(s)
    d0 = np.full(cr.shape, cr.n_elec / (cr.ng * cr.dV))
    exc, vxc, vh = go.lda_hartree(d0)
    v = go.ion_potential() + vh + vxc
    s.close()
    assert np.max(np.abs(v.ravel()[g["sample"]] - g["v_sample"])) < 1e-12
    return g, cr, b, v


@pytest.mark.parametrize("route", ["tridiag", "ldl"])
def test_fp64_pass_matches_reference_at_1024_electrons(jit8, route):
    from lresdft_gb300 import LResGPU
    g, cr, b, v = jit8
    s = LResGPU(b, cr.pos, R_w=8.0, M=64, precision="fp64", route=route)
    assert np.array_equal(s.nW, g["nW"])
    s.set_potential(v)
    dens, N, eb = s.pole_pass(float(g["mu"]), float(g["e_lo"]))
    err_d = float(np.max(np.abs(dens.ravel()[g["sample"]] - g["dens_sample"])))
    err_e = abs(eb - float(g["eband"]))
    print(route, "density", err_d, "band energy", err_e, "N", N)
    assert err_d < 1e-10 and err_e < 1e-9
    assert abs(N - cr.n_elec) < 1e-6
    s.close()


def test_mixed_pass_within_gate_at_1024_electrons(jit8):
    from lresdft_gb300 import LResGPU
    g, cr, b, v = jit8
    s = LResGPU(b, cr.pos, R_w=8.0, M=64, precision="mixed")
    assert s.route == "tridiag"
    s.set_potential(v)
    dens, N, eb = s.pole_pass(float(g["mu"]), float(g["e_lo"]))
    err_e = abs(eb - float(g["eband"])) / cr.n_elec
    err_d = float(np.max(np.abs(dens.ravel()[g["sample"]] - g["dens_sample"])))
    print("mixed: band energy per electron", err_e, "density", err_d, "count", abs(N - cr.n_elec))
    assert err_e < 2e-7 and err_d < 1e-6
    assert abs(N - cr.n_elec) / cr.n_elec < 1e-6
    s.close()


def test_mixed_tensor_core_standard_form_at_1024_electrons(jit8):
    """The mixed pass with the standard form on the tensor cores (tcgen05, 3xTF32): within the
    same gates as the SIMT standard form."""
    from lresdft_gb300 import LResGPU
    g, cr, b, v = jit8
    s = LResGPU(b, cr.pos, R_w=8.0, M=64, precision="mixed")
    s.set_standard_form("tensor")
    s.set_potential(v)
    dens, N, eb = s.pole_pass(float(g["mu"]), float(g["e_lo"]))
    err_e = abs(eb - float(g["eband"])) / cr.n_elec
    err_d = float(np.max(np.abs(dens.ravel()[g["sample"]] - g["dens_sample"])))
    print("mixed, tensor-core standard form: band energy per electron", err_e, "density", err_d)
    assert err_e < 2e-7 and err_d < 1e-6
    assert abs(N - cr.n_elec) / cr.n_elec < 1e-6
    s.close()


def test_density_call_reproduces_reference_cold_call(jit8):
    """The drop-in protocol at 1024 electrons: a cold density() call finds the reference's
    e_lo and mu and its density (FP64)."""
    from lresdft_gb300 import LResGPU
    g, cr, b, v = jit8
    s = LResGPU(b, cr.pos, R_w=8.0, M=64, precision="fp64")
    dens, eb, mu = s.density(v)
    print("cold call: mu", mu, "passes", s.passes, "e_lo", s.e_lo)
    assert abs(s.e_lo - float(g["e_lo"])) < 1e-9
    assert abs(mu - float(g["mu"])) < 1e-9
    assert abs(eb - float(g["eband"])) < 1e-8
    assert np.max(np.abs(dens.ravel()[g["sample"]] - g["dens_sample"])) < 1e-9
    s.close()
