"""Host logic of the solver that runs without a GPU: the windows the GPU solves (identical
windows merged, atoms that touch no owned point first) and the trace-row factor of the
owned-row Gram matrix."""
import numpy as np
import pytest

from golden_util import crystal, load


@pytest.fixture(scope="module")
def cubic3():
    from lresdft_gb300 import system
    g = load("cubic3")
    cr = crystal(g)
    return g, cr, system.LCAOBasis(cr)


def _windows(b, cr, R_w):
    from oracle import lrft_oracle as O
    windows, own, _ = O.window_setup(b, cr.pos, R_w)
    return windows, own


def test_solved_windows_reorder_whole_atoms(cubic3):
    from lresdft_gb300.solver import solved_windows
    g, cr, b = cubic3
    windows, own = _windows(b, cr, float(g["R_w"]))
    cw, cown, ctx_of = solved_windows(b, windows, own)
    assert len(cw) == len(windows) and np.array_equal(ctx_of, np.arange(len(windows)))
    aof = np.asarray(b.atom_of_fn)
    moved = 0
    for W, Wc, o in zip(windows, cw, cown):
        assert np.array_equal(np.sort(Wc), np.sort(W))               # a permutation of W
        atoms = aof[Wc]
        starts = np.flatnonzero(np.r_[True, atoms[1:] != atoms[:-1]])
        assert len(np.unique(atoms)) == len(starts)                 # atoms stay contiguous
        for s0 in starts:                                           # in function order
            f = Wc[s0:s0 + np.sum(atoms == atoms[s0])]
            assert np.all(np.diff(f) == 1)
        F = b.Xr[o][:, Wc].toarray()
        touch = np.abs(F).sum(axis=0) > 0
        first = np.flatnonzero(touch)[0]
        assert not touch[:first].any()
        # every function of a touching atom comes after every function of a non-touching one
        t_atoms = set(aof[Wc][touch])
        is_t = np.array([a in t_atoms for a in aof[Wc]])
        assert np.all(np.diff(is_t.astype(int)) >= 0)
        moved += first > 0
    assert moved > 0                                                # some windows reordered


def test_solved_windows_merge_identical():
    """2x2x2 cell at R_w = 8: every window is the whole cell; one solved window owns the grid."""
    from lresdft_gb300 import system
    from lresdft_gb300.solver import solved_windows
    g = load("jit2")
    cr = crystal(g)
    b = system.LCAOBasis(cr)
    windows, own = _windows(b, cr, 8.0)
    cw, cown, ctx_of = solved_windows(b, windows, own)
    assert len(cw) == 1 and np.all(ctx_of == 0)
    assert np.array_equal(cown[0], np.arange(cr.ng))
    cw2, cown2, ctx2 = solved_windows(b, windows, own, merge=False)
    assert len(cw2) == len(windows)


@pytest.mark.parametrize("pivoted", [True, False, "broken"])
def test_trace_factor(monkeypatch, pivoted):
    """R^T R = K with rank(K) rows and zero leading columns, by the pivoted Cholesky and by
    its eigendecomposition fallback; a zero column inside the touching block stays zero."""
    from scipy.linalg import lapack
    from lresdft_gb300.solver import trace_factor
    if pivoted is False:
        monkeypatch.setattr(lapack, "dpstrf", None, raising=False)
    elif pivoted == "broken":
        def old_wrapper(a):
            raise TypeError("no tol keyword")
        monkeypatch.setattr(lapack, "dpstrf", old_wrapper, raising=False)
        pivoted = False
    rng = np.random.default_rng(1)
    n, c0, m = 40, 9, 25
    F = np.zeros((m, n))
    F[:, c0:] = rng.normal(size=(m, n - c0))
    F[:, 20] = 0.0
    K = F.T @ F
    R = trace_factor(K)
    assert R.shape[0] == min(m, n - c0 - 1)
    assert np.all(R[:, :c0] == 0.0)
    # the pivoted factor never picks a zero pivot; the eigenvectors carry rounding there
    assert np.max(np.abs(R[:, 20])) <= (0.0 if pivoted else 1e-12 * np.max(np.abs(R)))
    assert np.max(np.abs(R.T @ R - K)) < 1e-12 * np.max(np.abs(K))
    assert trace_factor(np.zeros((5, 5))).shape == (0, 5)


def test_trace_factor_on_owned_rows():
    """Owned-row Gram matrices of the 3x3x3 golden crystal's windows: the trace over the
    factor's rows equals the trace over the owned points for a resolvent (z S - H)^-1,
    to 1e-12 relative."""
    from scipy import linalg
    from lresdft_gb300 import system
    from lresdft_gb300.solver import trace_factor
    from oracle import lrft_oracle as O
    g = load("cubic3")
    cr = crystal(g)
    b = system.LCAOBasis(cr)
    windows, own, _ = O.window_setup(b, cr.pos, float(g["R_w"]))
    H = b.H(g["v"].ravel())
    z = O.nodes(64, float(g["cold_mu"]), float(g["cold_elo"]))[0][5]
    for W, o in list(zip(windows, own))[:6]:
        F = b.Xr[o][:, W].toarray()
        K = F.T @ F
        R = trace_factor(K)
        assert R.shape[0] <= min(len(o), len(W))
        Ai = linalg.inv(z * b.S[W][:, W].toarray() - H[W][:, W].toarray())
        ex = np.trace(Ai @ K)
        assert abs(np.trace(Ai @ (R.T @ R)) - ex) < 1e-12 * abs(ex)


@pytest.mark.parametrize("kw", [dict(M=63), dict(M=0), dict(precision="fp32"), dict(R_w=0.0),
                                dict(tile_config=7), dict(tile_config="fast")])
def test_solver_rejects_bad_arguments(kw):
    """Constructor arguments are checked before any device work (ValueError, as the
    reference's own argument errors)."""
    from lresdft_gb300 import LResGPU, system
    cr = system.cubic_h2((1, 1, 1), pts_per_cell=8)
    b = system.LCAOBasis(cr)
    args = dict(R_w=8.0, M=64, precision="fp64", tile_config=None)
    args.update(kw)
    with pytest.raises(ValueError):
        LResGPU(b, cr.pos, **args)
