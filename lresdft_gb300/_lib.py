"""ctypes binding of liblres_gb300.so (include/lres_gb300.h).

The library is built in-tree by ``lresdft_gb300.build``; importing this module
loads it and raises if it is missing — there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblres_gb300.so")

LRES_FP64, LRES_MIXED = 0, 1
LRES_ROUTE_LDL, LRES_ROUTE_TRIDIAG = 0, 1
LRES_SF_SIMT, LRES_SF_TENSOR = 0, 1
ERRORS = {-22: "EINVAL", -12: "ENOMEM", -5: "ECUDA", -33: "ENUMERIC", -71: "ESTATE"}

EXPORTS = ("lres_version", "lres_last_error", "lres_ctx_create", "lres_ctx_destroy", "lres_set_potential",
           "lres_set_hamiltonian_csr", "lres_pass", "lres_pass_async", "lres_status", "lres_density_ptr", "lres_autotune",
           "lres_set_route", "lres_get_route", "lres_timings", "lres_window_sums", "lres_inertia", "lres_min_eig",
           "lres_voronoi_owner", "lres_lda_xc", "lres_hartree", "lres_ion_potential", "lres_inertia_noalloc",
           "lres_set_windows", "lres_window_ptrs", "lres_adjoint", "lres_owned_gram", "lres_set_trace_rows",
           "lres_basis_build", "lres_basis_fetch", "lres_basis_free", "lres_basis_tabulate",
           "lres_ks_density", "lres_set_standard_form_kernel", "lres_get_standard_form_kernel")


class LResError(RuntimeError):
    """A failed call of the C ABI (code and message of lres_last_error)."""

    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class NumericError(LResError):
    """LRES_ENUMERIC: a zero / non-finite pivot in some window factorisation."""


P64 = C.POINTER(C.c_int64)
PD = C.POINTER(C.c_double)


class SystemDesc(C.Structure):
    _fields_ = [("nb", C.c_int64), ("shape", C.c_int64 * 3), ("cell", C.c_double * 3), ("dV", C.c_double),
                ("Xp", P64), ("Xi", P64), ("Xv", PD),
                ("Sp", P64), ("Si", P64), ("Sv", PD),
                ("Tp", P64), ("Ti", P64), ("Tv", PD),
                ("ngroups", C.c_int64), ("gptr", P64),
                ("nwin", C.c_int64), ("Wflat", P64), ("Woff", P64), ("Oflat", P64), ("Ooff", P64)]


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} not built: run `python -m lresdft_gb300.build` (no CPU fallback)")
    lib = C.CDLL(LIB_PATH)
    vp, i32, i64, dbl = C.c_void_p, C.c_int, C.c_int64, C.c_double
    sig = {
        "lres_version": (C.c_char_p, []),
        "lres_last_error": (C.c_char_p, []),
        "lres_ctx_create": (i32, [C.POINTER(vp), C.POINTER(SystemDesc), i32, i32, vp]),
        "lres_ctx_destroy": (i32, [vp]),
        "lres_set_potential": (i32, [vp, vp, i32, vp]),
        "lres_set_hamiltonian_csr": (i32, [vp, P64, P64, PD, vp]),
        "lres_pass": (i32, [vp, dbl, dbl, vp, i32, PD, vp]),
        "lres_pass_async": (i32, [vp, dbl, dbl, vp, vp]),
        "lres_status": (i32, [vp, C.POINTER(C.c_int32), vp]),
        "lres_density_ptr": (i32, [vp, C.POINTER(C.c_void_p)]),
        "lres_autotune": (i32, [vp, dbl, dbl, C.c_int32, C.POINTER(C.c_int32), PD, vp]),
        "lres_set_route": (i32, [vp, C.c_int32, vp]),
        "lres_get_route": (i32, [vp, C.POINTER(C.c_int32)]),
        "lres_timings": (i32, [vp, PD, i32]),
        "lres_window_sums": (i32, [vp, PD, PD]),
        "lres_inertia": (i32, [vp, dbl, C.POINTER(C.c_int32), C.POINTER(i64), vp]),
        "lres_min_eig": (i32, [vp, dbl, dbl, dbl, PD, vp]),
        "lres_voronoi_owner": (i32, [P64, PD, i64, PD, C.POINTER(C.c_int32)]),
        "lres_lda_xc": (i32, [vp, vp, vp, vp, vp]),
        "lres_hartree": (i32, [vp, vp, vp, vp]),
        "lres_ion_potential": (i32, [vp, i64, PD, PD, PD, vp, vp]),
        "lres_inertia_noalloc": (i32, [C.c_int32, vp, vp, vp, vp, dbl, vp, C.c_int32, vp]),
        "lres_set_windows": (i32, [vp, vp, vp, i32, vp]),
        "lres_window_ptrs": (i32, [vp, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
        "lres_adjoint": (i32, [vp, dbl, dbl, vp, i32, vp, vp, i32, PD, vp]),
        "lres_owned_gram": (i32, [vp, vp, i32, vp]),
        "lres_set_trace_rows": (i32, [vp, vp, vp, vp]),
        "lres_basis_build": (i32, [C.POINTER(vp), i64, P64, P64, P64, PD, P64, dbl, dbl, dbl, i32, P64]),
        "lres_basis_fetch": (i32, [vp, P64, P64, PD, P64, P64, PD, P64, P64, PD, P64, P64, PD]),
        "lres_basis_free": (i32, [vp]),
        "lres_basis_tabulate": (i32, [i64, PD, C.POINTER(C.c_int32), C.POINTER(C.c_int32), PD, P64, PD, dbl, dbl,
                                      dbl, P64, P64, PD]),
        "lres_ks_density": (i32, [i64, P64, P64, PD, P64, P64, PD, i64, P64, P64, PD, C.c_int32, PD, PD, PD]),
        "lres_set_standard_form_kernel": (i32, [vp, C.c_int32]),
        "lres_get_standard_form_kernel": (i32, [vp, C.POINTER(C.c_int32)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype, f.argtypes = res, args
    return lib


lib = _load()


def check(rc):
    if rc:
        msg = lib.lres_last_error().decode(errors="replace")
        if rc == -33:
            raise NumericError(rc, msg)
        raise LResError(rc, msg)
    return rc


def ptr64(a):
    return a.ctypes.data_as(P64)


def ptrd(a):
    return a.ctypes.data_as(PD)


def i64(a):
    return np.ascontiguousarray(a, dtype=np.int64)


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def voronoi_owner(shape, cell, centres):
    """Nearest-centre ownership of every grid point (GPU)."""
    shape = i64(shape)
    cell = f64(cell)
    centres = f64(centres).reshape(-1, 3)
    owner = np.empty(int(np.prod(shape)), np.int32)
    check(lib.lres_voronoi_owner(ptr64(shape), ptrd(cell), centres.shape[0], ptrd(centres),
                                 owner.ctypes.data_as(C.POINTER(C.c_int32))))
    return owner


def basis_tabulate(pos, s_exps, p_exps, shape, cell, dx, rcut, dV):
    """Grid basis of every atom tabulated on the GPU (lres_basis_tabulate): per atom the
    points within rcut in cube order and the normalised s / p values.  s_exps, p_exps:
    one sequence of exponents per atom.  Returns (cnt, idx, val) in the layout of
    basis_matrices' inputs."""
    pos = f64(pos).reshape(-1, 3)
    nat = pos.shape[0]
    ns = np.array([len(e) for e in s_exps], np.int32)
    npp = np.array([len(e) for e in p_exps], np.int32)
    exps = f64([x for a in range(nat) for x in list(s_exps[a]) + list(p_exps[a])])
    shape, cell = i64(shape), f64(cell)
    cnt = np.zeros(nat, np.int64)
    i32p = C.POINTER(C.c_int32)
    args = (nat, ptrd(pos), ns.ctypes.data_as(i32p), npp.ctypes.data_as(i32p), ptrd(exps), ptr64(shape), ptrd(cell),
            float(dx), float(rcut), float(dV), ptr64(cnt))
    check(lib.lres_basis_tabulate(*args, None, None))
    nf = ns.astype(np.int64) + 3 * npp
    idx = np.empty(int(cnt.sum()), np.int64)
    val = np.empty(int((cnt * nf).sum()), np.float64)
    check(lib.lres_basis_tabulate(*args, ptr64(idx), ptrd(val)))
    return cnt, idx, val


def basis_matrices(gptr, cnt, idx, val, shape, dV, t_diag, t_off, nthreads=0):
    """Host assembly of the grouped grid basis (lres_basis_build): returns the CSC arrays
    of X (columns = functions), the CSR arrays of X, S and T, each (indptr, indices, data)."""
    gptr, cnt, idx, val, shape = i64(gptr), i64(cnt), i64(idx), f64(val), i64(shape)
    ngroups = len(cnt)
    h = C.c_void_p()
    nnz = np.zeros(3, np.int64)
    check(lib.lres_basis_build(C.byref(h), ngroups, ptr64(gptr), ptr64(cnt), ptr64(idx), ptrd(val), ptr64(shape),
                               float(dV), float(t_diag), float(t_off), int(nthreads), ptr64(nnz)))
    try:
        nb, ng = int(gptr[-1]), int(np.prod(shape))
        out = []
        for n_ptr, n in ((nb + 1, nnz[0]), (ng + 1, nnz[0]), (nb + 1, nnz[1]), (nb + 1, nnz[2])):
            out.append((np.empty(n_ptr, np.int64), np.empty(int(n), np.int64), np.empty(int(n), np.float64)))
        args = [f(a) for t in out for f, a in zip((ptr64, ptr64, ptrd), t)]
        check(lib.lres_basis_fetch(h, *args))
    finally:
        lib.lres_basis_free(h)
    return out
