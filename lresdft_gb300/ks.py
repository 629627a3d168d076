"""Dense Kohn-Sham LCAO on the GPU: the reference's ks_lcao (lrft/lcao3d.py:110-117) and its
native ks_density (src/lrft_cpp.cpp:235-284), through lres_ks_density.  The oracle side of
the identity LRes(R_w >= cell) = KS; the window solve is LResGPU."""
import numpy as np

from . import _lib
from .system import csr64


def ks_lcao(basis, v):
    """(density on the grid, band energy, the lowest nocc + 1 eigenvalues) of H(v), S."""
    cr = basis.cr
    nocc = cr.n_elec // 2
    Hp, Hi, Hv = csr64(basis.H(v))
    Sp, Si, Sv = csr64(basis.S)
    Xp, Xi, Xv = csr64(basis.Xr)
    dens = np.empty(cr.ng)
    w = np.empty(nocc + 1)
    eb = np.zeros(1)
    _lib.check(_lib.lib.lres_ks_density(basis.nb, _lib.ptr64(Hp), _lib.ptr64(Hi), _lib.ptrd(Hv), _lib.ptr64(Sp),
                                        _lib.ptr64(Si), _lib.ptrd(Sv), cr.ng, _lib.ptr64(Xp), _lib.ptr64(Xi),
                                        _lib.ptrd(Xv), int(nocc), _lib.ptrd(dens), _lib.ptrd(w), _lib.ptrd(eb)))
    return dens.reshape(cr.shape), float(eb[0]), w
