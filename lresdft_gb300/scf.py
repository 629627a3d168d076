"""SCF driver with the LDA and FFT-Hartree steps on the GPU.

``scf_lcao`` follows lrft/lcao3d.py:237-284 step for step (Pulay/DIIS with
ndiis=6, mix=0.4, clamp at 1e-12, renormalisation, Harris-Foulkes energy at the
input density of the last step); the potential v = v_ion + v_H[n] + v_xc[n] is
formed by the sm_103a kernels of liblres_gb300 (lres_lda_xc, lres_hartree,
lres_ion_potential).  The solver is any object with ``density(v)``; with an
``LResGPU`` solver its context also supplies the grid kernels.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np
import torch

from . import _lib


class GridOps:
    """Device buffers and the grid kernels of one crystal (needs an LResGPU context)."""

    def __init__(self, solver):
        self.s = solver
        self.cr = solver.b.cr
        ng = self.cr.ng
        self.dev = torch.device("cuda", torch.cuda.current_device())
        self.d_dens = torch.empty(ng, dtype=torch.float64, device=self.dev)
        self.d_exc = torch.empty_like(self.d_dens)
        self.d_vxc = torch.empty_like(self.d_dens)
        self.d_vh = torch.empty_like(self.d_dens)

    def _stream(self):
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)

    def ion_potential(self):
        cr = self.cr
        out = torch.empty(cr.ng, dtype=torch.float64, device=self.dev)
        pos = _lib.f64(cr.pos).ravel()
        Z = _lib.f64(cr.Z)
        rc = _lib.f64(cr.atom_rc)
        _lib.check(_lib.lib.lres_ion_potential(self.s._ctx, len(Z), _lib.ptrd(pos), _lib.ptrd(Z), _lib.ptrd(rc),
                                               out.data_ptr(), self._stream()))
        return out.cpu().numpy().reshape(cr.shape)

    def lda_hartree(self, dens):
        """(exc, vxc, vh) of a host density, computed on the GPU."""
        self.d_dens.copy_(torch.from_numpy(np.ascontiguousarray(dens, dtype=np.float64).ravel()))
        st = self._stream()
        _lib.check(_lib.lib.lres_lda_xc(self.s._ctx, self.d_dens.data_ptr(), self.d_exc.data_ptr(),
                                        self.d_vxc.data_ptr(), st))
        _lib.check(_lib.lib.lres_hartree(self.s._ctx, self.d_dens.data_ptr(), self.d_vh.data_ptr(), st))
        sh = self.cr.shape
        return (self.d_exc.cpu().numpy().reshape(sh), self.d_vxc.cpu().numpy().reshape(sh),
                self.d_vh.cpu().numpy().reshape(sh))


def scf_lcao(cr, solver, tol=1e-6, maxiter=60, mix=0.4, ndiis=6, verbose=False, dens0=None, grid=None,
             vion=None, step_times=None):
    t0 = time.perf_counter()
    grid = GridOps(solver) if grid is None else grid
    vion = grid.ion_potential() if vion is None else vion
    dens = np.full(cr.shape, cr.n_elec / (cr.ng * cr.dV)) if dens0 is None else dens0.copy()
    hist_n, hist_r = [], []
    converged = False
    for it in range(1, maxiter + 1):
        ts = time.perf_counter()
        exc, vxc, vh = grid.lda_hartree(dens)
        v = vion + vh + vxc
        out = solver.density(v)
        nout, eband = out[0], out[1]
        resid = nout - dens
        err = np.sum(np.abs(resid)) * cr.dV / cr.n_elec
        if verbose:
            print(f"  it {it:2d} |dn|/N = {err:.2e}  ({time.perf_counter() - ts:.2f}s)", flush=True)
        if err < tol:
            converged = True
            if step_times is not None:
                step_times.append(time.perf_counter() - ts)
            break
        hist_n.append(dens.copy())
        hist_r.append(resid.copy())
        if len(hist_n) > ndiis:
            hist_n.pop(0)
            hist_r.pop(0)
        k = len(hist_n)
        if k > 1:
            Bm = np.empty((k + 1, k + 1))
            Bm[:k, :k] = [[np.vdot(ri, rj) for rj in hist_r] for ri in hist_r]
            Bm[k, :k] = Bm[:k, k] = 1.0
            Bm[k, k] = 0.0
            rhs = np.zeros(k + 1)
            rhs[k] = 1.0
            coef = np.linalg.lstsq(Bm, rhs, rcond=None)[0][:k]
            dens = sum(c * h for c, h in zip(coef, hist_n)) + mix * sum(c * r for c, r in zip(coef, hist_r))
        else:
            dens = dens + mix * resid
        dens = np.maximum(dens, 1e-12)
        dens *= cr.n_elec / (dens.sum() * cr.dV)
        if step_times is not None:
            step_times.append(time.perf_counter() - ts)
    exc, vxc, vh = grid.lda_hartree(dens)
    E_H = 0.5 * np.sum(dens * vh) * cr.dV
    E_xc = np.sum(dens * exc) * cr.dV
    E = eband - np.sum((vh + vxc) * dens) * cr.dV + E_H + E_xc
    return dict(energy=E, density=nout, iterations=it, time=time.perf_counter() - t0, converged=converged,
                dens_in=dens, eband=eband, last=out, E_H=E_H, E_xc=E_xc)
