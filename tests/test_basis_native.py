"""Host assembly of the grid basis (lres_basis_build) against the scipy.sparse assembly the
reference uses (lrft/lcao3d.py:80-96): X (CSC and CSR), S = X^T X dV, T = X^T T_FD X dV.

Bit for bit where no atom's tabulation cube wraps onto one grid point three or more times;
where it does (2x2x2 cells: up to 8 periodic images of a point), the images are summed in
tabulation order, while scipy's order is its sort's, and the two differ in the last bit."""
import numpy as np
import pytest

from golden_util import check_basis, crystal, load


def _same(A, B, exact=True):
    A, B = A.tocsr(), B.tocsr()
    A.sort_indices()
    B.sort_indices()
    assert A.shape == B.shape and A.nnz == B.nnz
    assert np.array_equal(A.indptr, B.indptr) and np.array_equal(A.indices, B.indices)
    if exact:
        assert np.array_equal(A.data, B.data)
    else:
        assert np.max(np.abs(A.data - B.data)) <= 1e-15 * np.max(np.abs(B.data))


def _pair(cr, **kw):
    from lresdft_gb300 import system
    return system.LCAOBasis(cr, **kw), system.LCAOBasis(cr, assembly="scipy", **kw)


@pytest.mark.parametrize("name,exact", [("cubic3", True), ("jit2", False)])
def test_native_equals_scipy_on_golden_systems(name, exact):
    g = load(name)
    cr = crystal(g)
    bn, bs = _pair(cr)
    for attr in ("X", "Xr", "S", "T"):
        _same(getattr(bn, attr), getattr(bs, attr), exact)
    check_basis(bn, g)


def test_mixed_function_counts_and_threads():
    """Atoms with 3, 6 and 7 functions (atom_exps), a jittered 3x3x3 cell; the result does
    not depend on the number of threads."""
    from lresdft_gb300 import system
    cr = system.jittered_h2((3, 3, 3), a=4.5, bond=1.4, pts_per_cell=8, jitter=0.1, seed=5)
    kinds = [((1.0, 0.3, 0.12), ()), ((1.0, 0.3, 0.12), (0.5,)), ((1.1, 0.4, 0.15, 0.06), (0.45,))]
    atom_exps = [kinds[a % 3] for a in range(len(cr.pos))]
    bn, bs = _pair(cr, atom_exps=atom_exps)
    assert set(np.diff(bn.atom_fn_ptr)) == {3, 6, 7}
    for attr in ("X", "Xr", "S", "T"):
        _same(getattr(bn, attr), getattr(bs, attr))
    b1 = system.LCAOBasis(cr, atom_exps=atom_exps, nthreads=1)
    b3 = system.LCAOBasis(cr, atom_exps=atom_exps, nthreads=3)
    for attr in ("S", "T", "Xr"):
        _same(getattr(b1, attr), getattr(b3, attr))
        _same(getattr(b1, attr), getattr(bn, attr))


def test_two_point_axis_stencil():
    """A grid axis of two points: the +1 and -1 neighbours coincide and the stencil entry
    is their sum, as in scipy's COO assembly of T_FD."""
    from lresdft_gb300 import system
    a = 4.5
    cr = system.Crystal(np.array([[0.3, 2.1, 2.2], [0.4, 2.3, 3.5]]), np.ones(2), np.array([a / 8 * 2, a, a]),
                        (2, 8, 8), 1.0)
    bn, bs = _pair(cr, rcut=2.0)
    for attr in ("X", "Xr", "S", "T"):
        _same(getattr(bn, attr), getattr(bs, attr), exact=False)


def test_invalid_input_is_reported():
    import ctypes as C
    from lresdft_gb300 import _lib
    gptr = np.array([0, 9], np.int64)          # nine functions in one group
    cnt = np.array([1], np.int64)
    idx = np.array([0], np.int64)
    with pytest.raises(_lib.LResError, match="1..8"):
        _lib.basis_matrices(gptr, cnt, idx, np.ones(9), (2, 2, 2), 1.0, 1.0, -1.0)
    with pytest.raises(_lib.LResError, match="out of range"):
        _lib.basis_matrices(np.array([0, 1]), cnt, np.array([8]), np.ones(1), (2, 2, 2), 1.0, 1.0, -1.0)
    h = C.c_void_p()
    assert _lib.lib.lres_basis_build(C.byref(h), 0, None, None, None, None, None, 1.0, 1.0, -1.0, 1, None) == -22


def test_one_and_eight_function_atoms_and_many_threads():
    """Atoms with a single s function and with eight (five s + one p shell), the widest value
    lane count; 64 threads (more than the host has) give the same matrices as one."""
    from lresdft_gb300 import system
    cr = system.jittered_h2((2, 2, 2), a=5.0, bond=1.4, pts_per_cell=8, jitter=0.1, seed=2)
    kinds = [((0.8,), ()), ((1.5, 0.9, 0.5, 0.25, 0.1), (0.4,))]
    atom_exps = [kinds[a % 2] for a in range(len(cr.pos))]
    bn, bs = _pair(cr, atom_exps=atom_exps)
    assert set(np.diff(bn.atom_fn_ptr)) == {1, 8}
    for attr in ("X", "Xr", "S", "T"):
        _same(getattr(bn, attr), getattr(bs, attr), exact=False)
    b1 = system.LCAOBasis(cr, atom_exps=atom_exps, nthreads=1)
    b64 = system.LCAOBasis(cr, atom_exps=atom_exps, nthreads=64)
    for attr in ("X", "Xr", "S", "T"):
        _same(getattr(b1, attr), getattr(b64, attr))


def test_tabulation_and_dense_ks_argument_checks():
    """Host-side argument checks of the GPU entry points (no device work): the tabulation
    option of LCAOBasis, lres_basis_tabulate, lres_ks_density and the standard-form switch."""
    import ctypes as C
    from lresdft_gb300 import _lib, system
    g = load("cubic3")
    cr = crystal(g)
    with pytest.raises(ValueError, match="tabulation"):
        system.LCAOBasis(cr, tabulation="cpu")
    with pytest.raises(ValueError, match="native"):
        system.LCAOBasis(cr, tabulation="gpu", assembly="scipy")
    cnt = np.zeros(1, np.int64)
    shape = np.array([4, 4, 4], np.int64)
    cell = np.array([4.0, 4.0, 4.0])
    ns = np.array([3], np.int32)
    npp = np.array([1], np.int32)
    exps = np.array([1.0, 0.3, 0.12, 0.5])
    pos = np.zeros(3)
    i32p = C.POINTER(C.c_int32)
    args = [1, _lib.ptrd(pos), ns.ctypes.data_as(i32p), npp.ctypes.data_as(i32p), _lib.ptrd(exps), _lib.ptr64(shape),
            _lib.ptrd(cell), 1.0, 5.5, 1.0, _lib.ptr64(cnt)]
    bad = list(args)
    bad[0] = 0                                            # no atoms
    assert _lib.lib.lres_basis_tabulate(*bad, None, None) == -22
    bad = list(args)
    bad[7] = -1.0                                         # dx <= 0
    assert _lib.lib.lres_basis_tabulate(*bad, None, None) == -22
    ns9 = np.array([9], np.int32)                         # nine functions on one atom
    bad = list(args)
    bad[2] = ns9.ctypes.data_as(i32p)
    assert _lib.lib.lres_basis_tabulate(*bad, None, None) == -22
    assert b"1..8" in _lib.lib.lres_last_error()
    idx = np.zeros(1, np.int64)
    assert _lib.lib.lres_basis_tabulate(*args, _lib.ptr64(idx), None) == -22     # idx without val
    z = np.zeros(2, np.int64)
    d = np.zeros(2)
    assert _lib.lib.lres_ks_density(1, _lib.ptr64(z), _lib.ptr64(z), _lib.ptrd(d), _lib.ptr64(z), _lib.ptr64(z),
                                    _lib.ptrd(d), 1, _lib.ptr64(z), _lib.ptr64(z), _lib.ptrd(d), 1, _lib.ptrd(d),
                                    _lib.ptrd(d), _lib.ptrd(d)) == -22   # nocc >= nb
    assert _lib.lib.lres_set_standard_form_kernel(None, 1) == -22
