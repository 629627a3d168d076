"""Parity of the sm_103a path (through the C ABI) with the reference's own outputs
(tests/golden, produced by the reference code) and with the CPU oracle.

Tolerances: FP64 path 1e-10 on densities, 1e-9 on band energies (the reference's own
C++-vs-Python gate, tests/test_three_d.py:86-100) and 1e-10 Ha/electron on SCF
energies; mixed path (complex64 factor/solve + FP64 refinement-free sums) 2e-7
Ha/electron on energies."""
import numpy as np
import pytest

from golden_util import check_basis, crystal, load

pytestmark = pytest.mark.gpu

CASES = ["jit2", "cubic3"]


@pytest.fixture(scope="module")
def systems():
    from lresdft_gb300 import system
    out = {}
    for name in CASES:
        g = load(name)
        cr = crystal(g)
        b = system.LCAOBasis(cr)
        check_basis(b, g)
        out[name] = (g, cr, b)
    return out


def _copy_device(ptr, host):
    """Device-to-host copy of a raw device array of doubles (wrapped for torch through the
    CUDA array interface)."""
    import torch

    class _Dev:
        __cuda_array_interface__ = {"shape": (host.size,), "typestr": "<f8",
                                    "data": (int(ptr), False), "version": 3}
    torch.cuda.synchronize()
    host[:] = torch.as_tensor(_Dev(), device="cuda").cpu().numpy()


def _solver(b, cr, g, precision="fp64", **kw):
    from lresdft_gb300 import LResGPU
    return LResGPU(b, cr.pos, R_w=float(g["R_w"]), M=int(g["M"]), precision=precision, **kw)


@pytest.mark.parametrize("name", CASES)
def test_voronoi_and_windows_match_reference(systems, name):
    g, cr, b = systems[name]
    s = _solver(b, cr, g)
    assert np.array_equal(s.owner, g["owner"])
    assert np.array_equal(s.Wflat, g["Wflat"])
    s.close()


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("hpath", ["gpu", "csr"])
def test_single_pass_matches_reference_density(systems, name, hpath):
    """One pole pass at the reference's (mu, e_lo) reproduces its cold density call."""
    g, cr, b = systems[name]
    s = _solver(b, cr, g)
    v = g["v"].reshape(cr.shape)
    if hpath == "gpu":
        s.set_potential(v)
    else:
        s.set_hamiltonian(b.H(v))
    dens, N, eb = s.pole_pass(float(g["cold_mu"]), float(g["cold_elo"]))
    assert np.max(np.abs(dens - g["cold_dens"])) < 1e-10
    assert abs(eb - g["cold_eband"]) < 1e-9
    assert abs(N - cr.n_elec) < 1e-7
    s.close()


def _nonlocal_term(b, natoms, seed=7, k=2):
    """A separable nonlocal term of the GTH form, sum over atoms of B_a h_a B_a^T (projectors
    B_a on the atom's own functions, positive strengths h_a), as a CSR matrix over the basis."""
    from scipy import sparse
    rng = np.random.default_rng(seed)
    rows, cols, vals = [], [], []
    for a in range(natoms):
        f = np.flatnonzero(b.atom_of_fn == a)
        B = 0.3 * rng.standard_normal((len(f), k))
        V = B @ np.diag(rng.uniform(0.1, 0.5, k)) @ B.T
        V = 0.5 * (V + V.T)                             # exactly symmetric
        ii, jj = np.meshgrid(f, f, indexing="ij")
        rows.append(ii.ravel())
        cols.append(jj.ravel())
        vals.append(V.ravel())
    nb = len(b.atom_of_fn)
    return sparse.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(nb, nb))


@pytest.mark.parametrize("route", ["tridiag", "ldl"])
def test_nonlocal_hamiltonian_through_csr(systems, route):
    """A Hamiltonian that is not an LCAO H(v): H(v) plus a separable nonlocal term of the form
    a GTH pseudopotential adds (lrft/gth.py:105-232 assembles its H so), given through the CSR
    entry point (lres_set_hamiltonian_csr, the H argument of lrft_windows): one FP64 pass at the
    reference's (mu, e_lo) against the oracle's pole route on the same matrix, 1e-10 in the
    density and 1e-9 in the band energy."""
    from oracle import lrft_oracle as orc
    g, cr, b = systems["jit2"]
    v = g["v"].reshape(cr.shape)
    H = (b.H(v) + _nonlocal_term(b, len(cr.pos))).tocsr()
    H.sort_indices()
    mu, e_lo = float(g["cold_mu"]), float(g["cold_elo"])
    s = _solver(b, cr, g, route=route)
    s.set_hamiltonian(H)
    dens, N, eb = s.pole_pass(mu, e_lo)
    ref, Nr, Er = orc.pole_density(H, b.S, b.Xr, s.windows, s.own, cr.ng, cr.dV, mu, e_lo, s.M)
    s.close()
    own = np.concatenate(s.own)
    assert np.max(np.abs(dens[own] - ref[own])) < 1e-10
    assert abs(eb - Er) < 1e-9 and abs(N - Nr) < 1e-9
    assert abs(Nr - cr.n_elec) > 1e-3               # the term moved the electron count: H was used


@pytest.mark.parametrize("name", CASES)
def test_routes_agree(systems, name):
    """The tridiagonal route (the default) and the LDL^T route evaluate the same resolvent
    quadratic forms: FP64 densities within 1e-12, band energies within 1e-11, inertia counts
    equal; mixed precision: both within the 2e-7 Ha/electron gate of the reference, and the
    mixed density within 1e-6 of FP64 in L2 per electron."""
    g, cr, b = systems[name]
    v = g["v"].reshape(cr.shape)
    mu, e_lo = float(g["cold_mu"]), float(g["cold_elo"])
    sig = float(g["lam_min"].min()) + 0.05
    for precision in ("fp64", "mixed"):
        out = {}
        for route in ("ldl", "tridiag"):
            s = _solver(b, cr, g, precision, route=route)
            assert s.route == route
            s.set_potential(v)
            dens, N, eb = s.pole_pass(mu, e_lo)
            out[route] = (dens, N, eb, s.inertia(sig, per_window=True))
            s.close()
        a, t = out["ldl"], out["tridiag"]
        assert np.array_equal(a[3], t[3])
        if precision == "fp64":
            assert np.max(np.abs(a[0] - t[0])) < 1e-12 and abs(a[2] - t[2]) < 1e-11 and abs(a[1] - t[1]) < 1e-11
        else:
            for r in (a, t):
                assert abs(r[2] - g["cold_eband"]) / cr.n_elec < 2e-7
                assert np.sqrt(np.sum((r[0] - g["cold_dens"]) ** 2) * cr.dV) / cr.n_elec < 1e-6


def test_route_switch_keeps_results(systems):
    """lres_set_route on a context with a Hamiltonian: the tridiagonal form is rebuilt on the
    switch, and switching back and forth gives the same pass bit for bit."""
    g, cr, b = systems["cubic3"]
    mu, e_lo = float(g["cold_mu"]), float(g["cold_elo"])
    s = _solver(b, cr, g, "fp64", route="ldl")
    s.set_potential(g["v"].reshape(cr.shape))
    d0, N0, E0 = s.pole_pass(mu, e_lo)
    s.set_route("tridiag")
    d1, N1, E1 = s.pole_pass(mu, e_lo)
    s.set_route("ldl")
    d2, N2, E2 = s.pole_pass(mu, e_lo)
    s.set_route("tridiag")
    d3, N3, E3 = s.pole_pass(mu, e_lo)
    assert np.array_equal(d0, d2) and E0 == E2
    assert np.array_equal(d1, d3) and E1 == E3
    assert np.max(np.abs(d1 - g["cold_dens"])) < 1e-10
    s.close()


@pytest.mark.parametrize("name", CASES)
def test_pass_is_bitwise_reproducible(systems, name):
    g, cr, b = systems[name]
    s = _solver(b, cr, g)
    s.set_potential(g["v"].reshape(cr.shape))
    a = s.pole_pass(float(g["cold_mu"]), float(g["cold_elo"]))
    c = s.pole_pass(float(g["cold_mu"]), float(g["cold_elo"]))
    assert np.array_equal(a[0], c[0]) and a[1] == c[1] and a[2] == c[2]
    s.close()


@pytest.mark.parametrize("name", CASES)
def test_inertia_counts_bracket_window_minima(systems, name):
    g, cr, b = systems[name]
    s = _solver(b, cr, g)
    s.set_potential(g["v"].reshape(cr.shape))
    lm = g["lam_min"]
    below_lo = s.inertia(float(lm.min()) - 1e-7, per_window=True)
    assert below_lo.sum() == 0
    per = np.array([s.inertia(float(x) + 1e-7, per_window=True)[w] for w, x in enumerate(lm)])
    assert np.all(per >= 1)
    assert abs(s.min_eig(-1.0, 0.0, tol=1e-12) - lm.min()) < 1e-10
    s.close()


@pytest.mark.parametrize("name", CASES)
def test_density_protocol_matches_reference_calls(systems, name):
    """Cold call, warm call with a forced mu re-solve, and a warm call that keeps mu
    (the three calls of tests/golden/make_golden.py, reuse_vectors=False).  Without trace rows,
    so that the pass counts are the reference's (with them, the first warm pass after a re-solve
    runs over the trace rows and a kept mu costs that pass plus the density pass)."""
    g, cr, b = systems[name]
    s = _solver(b, cr, g, trace_rows=False)
    v = g["v"].reshape(cr.shape)
    n1, e1, mu1 = s.density(v)
    assert abs(s.e_lo - g["cold_elo"]) < 1e-9
    assert abs(mu1 - g["cold_mu"]) < 1e-9
    assert abs(e1 - g["cold_eband"]) < 1e-9
    assert np.max(np.abs(n1.ravel() - g["cold_dens"])) < 1e-10
    s.mu += 0.02
    n2, e2, mu2 = s.density(0.999 * v)
    assert abs(mu2 - g["warm_mu"]) < 1e-9
    assert abs(e2 - g["warm_eband"]) < 1e-9
    assert np.max(np.abs(n2.ravel() - g["warm_dens"])) < 1e-10
    p0 = s.passes
    n3, e3, mu3 = s.density(0.999 * v)
    assert s.passes - p0 == 1 and mu3 == mu2
    assert abs(e3 - g["keep_eband"]) < 1e-9
    assert np.max(np.abs(n3.ravel() - g["keep_dens"])) < 1e-10
    s.close()


@pytest.mark.parametrize("name", CASES)
def test_mixed_precision_density_within_gate(systems, name):
    g, cr, b = systems[name]
    s = _solver(b, cr, g, precision="mixed")
    v = g["v"].reshape(cr.shape)
    s.set_potential(v)
    dens, N, eb = s.pole_pass(float(g["cold_mu"]), float(g["cold_elo"]))
    ne = cr.n_elec
    assert abs(eb - g["cold_eband"]) / ne < 2e-7
    assert abs(N - ne) / ne < 1e-6
    assert np.sqrt(np.sum((dens - g["cold_dens"]) ** 2) * cr.dV) / ne < 1e-6
    n1, e1, mu1 = s.density(v)
    assert abs(e1 - g["cold_eband"]) / ne < 2e-7
    s.close()


@pytest.mark.parametrize("name", CASES)
def test_mixed_h_assembly_blocked_sums(systems, name):
    """The mixed context assembles H(v) from FP32 products with FP32 sums over blocks of 32
    common points per lane and FP64 sums of the blocks; the FP64 context in FP64.  Both
    against the host H(v) = T + X^T diag(v) X dV (lrft/lcao3d.py:98-100) window by window:
    FP64 to 1e-12 Ha, mixed to 1e-6 Ha (FP32 rounding of the basis values and the
    potential), with a mean error (the drift of long FP32 sums) below 1e-8 Ha."""
    from lresdft_gb300.autograd import window_matrices
    g, cr, b = systems[name]
    v = g["v"].reshape(cr.shape)
    Hhost = b.H(v).tocsr()
    errs = {}
    for precision in ("fp64", "mixed"):
        s = _solver(b, cr, g, precision=precision)
        s.set_potential(v)
        HW = window_matrices(s)[0].cpu().numpy()
        off = s.window_offsets
        d = []
        for w, W in enumerate(s.ctx_windows):
            n = len(W)
            blk = HW[off[w]:off[w + 1]].reshape(n, n, order="F")
            d.append((blk - Hhost[W][:, W].toarray()).ravel())
        errs[precision] = np.concatenate(d)
        s.close()
    assert np.max(np.abs(errs["fp64"])) < 1e-12
    assert np.max(np.abs(errs["mixed"])) < 1e-6
    assert abs(np.mean(errs["mixed"])) < 1e-8


def test_grid_kernels_match_oracle(systems):
    from lresdft_gb300.scf import GridOps
    from oracle import lrft_oracle as orc
    g, cr, b = systems["cubic3"]
    s = _solver(b, cr, g)
    go = GridOps(s)
    vion = go.ion_potential()
    assert np.max(np.abs(vion.ravel() - g["vion"])) < 1e-11
    rng = np.random.default_rng(3)
    dens = np.abs(rng.normal(size=cr.shape)) * 0.05 + 1e-3
    exc, vxc, vh = go.lda_hartree(dens)
    e0, v0 = orc.lda_xc(dens)
    assert np.max(np.abs(exc - e0)) < 1e-13 and np.max(np.abs(vxc - v0)) < 1e-13
    assert np.max(np.abs(vh - orc.hartree(cr, dens))) < 1e-12
    s.close()


@pytest.mark.parametrize("name", CASES)
def test_scf_energy_matches_reference(systems, name):
    """SCF against the reference's LRFTLCAOCpp(reuse_vectors=False) SCF converged to
    tol 1e-8: FP64 with the same tolerance to 1e-10 Ha/e; mixed precision (whose
    density carries ~1e-7 relative FP32 noise, so |dn|/N cannot reach 1e-8) to tol 1e-6,
    energy within 2e-7 Ha/e."""
    from lresdft_gb300.scf import scf_lcao
    g, cr, b = systems[name]
    for precision, tol, gate in (("fp64", 1e-8, 1e-10), ("mixed", 1e-6, 2e-7)):
        s = _solver(b, cr, g, precision)
        r = scf_lcao(cr, s, tol=tol)
        assert r["converged"]
        assert abs(r["energy"] - g["scf_energy"]) / cr.n_elec < gate, (precision, r["energy"], g["scf_energy"])
        s.close()


def test_scf_on_device_matches_host_path(systems):
    """The SCF loop on device tensors (potential, densities, residual histories, DIIS
    combination, clamp and renormalisation on the GPU; only the residual norm and the Gram
    matrix to the host) against the host loop that keeps the reference's numpy operations:
    the same iterations and energies within 1e-12 Ha/electron."""
    from lresdft_gb300.scf import scf_lcao
    g, cr, b = systems["cubic3"]
    out = {}
    for device in (True, False):
        s = _solver(b, cr, g, "fp64")
        out[device] = scf_lcao(cr, s, tol=1e-8, device=device)
        s.close()
    d, h = out[True], out[False]
    assert d["converged"] and h["converged"] and d["iterations"] == h["iterations"]
    assert abs(d["energy"] - h["energy"]) / cr.n_elec < 1e-12
    assert abs(d["energy"] - g["scf_energy"]) / cr.n_elec < 1e-10
    assert np.max(np.abs(d["density"] - h["density"])) < 1e-10


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("config", [0, 1, 2, 3, 4, 5])
def test_every_tile_configuration_matches_reference(systems, name, config):
    """Each compiled tile configuration of the LDL^T pole kernel, forced: FP64 to 1e-10 in
    density, mixed within the 2e-7 Ha/electron gate (configuration 4 of the mixed path runs
    the chunk products on the tensor cores with a 3xTF32 split)."""
    g, cr, b = systems[name]
    v = g["v"].reshape(cr.shape)
    for precision in ("fp64", "mixed"):
        s = _solver(b, cr, g, precision, route="ldl")
        s.autotune(0.0, -1.0, config=config)
        s.set_potential(v)
        dens, N, eb = s.pole_pass(float(g["cold_mu"]), float(g["cold_elo"]))
        if precision == "fp64":
            assert np.max(np.abs(dens - g["cold_dens"])) < 1e-10 and abs(eb - g["cold_eband"]) < 1e-9
        else:
            assert abs(eb - g["cold_eband"]) / cr.n_elec < 2e-7
        s.close()


@pytest.mark.parametrize("name", CASES)
def test_tensor_core_standard_form(systems, name):
    """The mixed standard form on the tensor cores (tcgen05, 3xTF32, 32-term chunks): the band
    energy within the 2e-7 Ha/electron gate of the reference and the density norm within 1e-6,
    like the SIMT kernels, and no tensor-core completion timeout (a timeout fails the pass).
    Its distance from the SIMT result is printed, not gated: the tensor core's accumulation of
    each chunk is less exact than the FP32 FMA chain (5e-8 Ha/electron on jit2, 4.9e-8 against
    5e-10 from the reference at 1024 electrons)."""
    g, cr, b = systems[name]
    v = g["v"].reshape(cr.shape)
    ne = cr.n_elec
    res = {}
    for kind in ("simt", "tensor"):
        s = _solver(b, cr, g, "mixed", route="tridiag")
        s.set_standard_form(kind)
        assert s.standard_form == kind
        s.set_potential(v)
        dens, N, eb = s.pole_pass(float(g["cold_mu"]), float(g["cold_elo"]))
        assert abs(eb - g["cold_eband"]) / ne < 2e-7
        assert np.sqrt(np.sum((dens - g["cold_dens"]) ** 2) * cr.dV) / ne < 1e-6
        res[kind] = (dens, eb)
        s.close()
    print(name, "tensor vs SIMT standard form, band energy per electron",
          abs(res["tensor"][1] - res["simt"][1]) / ne)


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("config", [0, 1, 2, 3, 4, 5])
def test_every_tridiagonal_configuration_matches_reference(systems, name, config):
    """Each configuration of the tridiagonal route, forced (reduction with the window in
    shared memory or in the L2-resident working copy; row application with resident rows
    or one row per thread; panel widths): FP64 to 1e-10 in density, mixed within the 2e-7
    Ha/electron gate and 1e-6 in the density norm, after the potential was set and again
    after a second potential (the T factors and row items follow the configuration)."""
    g, cr, b = systems[name]
    v = g["v"].reshape(cr.shape)
    ne = cr.n_elec
    for precision in ("fp64", "mixed"):
        s = _solver(b, cr, g, precision, route="tridiag")
        s.set_potential(0.5 * v)
        s.autotune(0.0, -1.0, config=config)
        s.set_potential(v)
        dens, N, eb = s.pole_pass(float(g["cold_mu"]), float(g["cold_elo"]))
        if precision == "fp64":
            assert np.max(np.abs(dens - g["cold_dens"])) < 1e-10 and abs(eb - g["cold_eband"]) < 1e-9
        else:
            assert abs(eb - g["cold_eband"]) / ne < 2e-7
            assert np.sqrt(np.sum((dens - g["cold_dens"]) ** 2) * cr.dV) / ne < 1e-6
        s.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_pass_captured_in_cuda_graph(systems, precision):
    """lres_set_potential (device v) + lres_pass_async captured once in a CUDA graph and
    replayed: the same N, E_band and density as the synchronous lres_pass, bit for bit."""
    import torch
    g, cr, b = systems["cubic3"]
    mu, e_lo = float(g["cold_mu"]), float(g["cold_elo"])
    s = _solver(b, cr, g, precision)
    dev = torch.device("cuda", torch.cuda.current_device())
    v = torch.from_numpy(g["v"].copy()).to(dev)
    s.set_potential_device(v.data_ptr())
    dens_ref, N_ref, E_ref = s.pole_pass(mu, e_lo)
    out = torch.zeros(2, dtype=torch.float64, device=dev)
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.graph(graph, stream=side):
        st = torch.cuda.current_stream().cuda_stream
        s.set_potential_device(v.data_ptr(), st)
        s.pass_async(mu, e_lo, out.data_ptr(), st)
    for _ in range(2):
        out.zero_()
        graph.replay()
        torch.cuda.synchronize()
        assert s.status() == 0
        N, E = out.cpu().numpy()
        assert N == N_ref and E == E_ref
        host = np.empty(cr.ng)
        _copy_device(s.density_device_ptr(), host)
        assert np.array_equal(host, dens_ref)
    s.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cell_windows_reproduce_published_energy(precision):
    """The reference's published setting with cell-centred windows (benchmarks/scaling_rigorous.py:36,
    results/scaling_rigorous.json, n=3): 27 H2 cells, a=6, 10 points per cell, rc=0.6, benchmark
    basis, windows on the cell centres with R_w=12.1, M=64, SCF tol 1e-6:
    E_LRes(54 e) = -15.746532895084757.  The published run used float32 vector reuse (~1e-9 Ha);
    FP64 within 5e-9 Ha, mixed within 2e-7 Ha/electron."""
    from lresdft_gb300 import LResGPU, system
    from lresdft_gb300.scf import scf_lcao
    cr = system.h2_crystal((3, 3, 3), a=6.0, pts_per_cell=10, rc=0.6)
    b = system.LCAOBasis(cr, rcut=4.5, s_exps=(1.2, 0.4, 0.15), p_exps=(0.5,))
    s = LResGPU(b, system.cell_centres((3, 3, 3), 6.0), R_w=12.1, M=64, precision=precision)
    # every cell lies within 10.4 bohr < R_w of every other: 27 whole-cell windows, solved once
    assert len(s.windows) == 27 and np.all(s.nW == b.nb) and len(s.ctx_windows) == 1
    r = scf_lcao(cr, s, tol=1e-6)
    assert r["converged"]
    err = abs(r["energy"] - (-15.746532895084757))
    print(precision, "iterations", r["iterations"], "energy error", err)
    assert err < (5e-9 if precision == "fp64" else 2e-7 * cr.n_elec)
    s.close()
