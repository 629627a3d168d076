"""SCF driver with the LDA and FFT-Hartree steps on the GPU.

``scf_lcao`` runs the SCF of lrft/lcao3d.py:237-284 (Pulay/DIIS over ndiis=6 histories,
mix=0.4, clamp at 1e-12, renormalisation, Harris-Foulkes energy at the input density of the
last step); the potential v = v_ion + v_H[n] + v_xc[n] is formed by the sm_103a kernels of
liblres_gb300 (lres_lda_xc, lres_hartree, lres_ion_potential).  With a solver that offers
``density_device`` (``LResGPU``) every grid array stays in device memory: the potential, the
solver's output density, the residual histories, the DIIS combination, the clamp and the
renormalisation; per iteration only the residual norm and the k x k Gram matrix of the
residuals (k <= ndiis) reach the host, where the small bordered DIIS system is solved.  Any
other solver object with ``density(v)`` takes the host path, which keeps the reference's
numpy operations.
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

    def ion_potential_device(self):
        """v_ion as a device tensor (ng,)."""
        cr = self.cr
        out = torch.empty(cr.ng, dtype=torch.float64, device=self.dev)
        pos = _lib.f64(cr.pos).ravel()
        Z = _lib.f64(cr.Z)
        rc = _lib.f64(cr.atom_rc)
        _lib.check(_lib.lib.lres_ion_potential(self.s._ctx, len(Z), _lib.ptrd(pos), _lib.ptrd(Z), _lib.ptrd(rc),
                                               out.data_ptr(), self._stream()))
        return out

    def lda_hartree_device(self, dens):
        """(exc, vxc, vh) of a device density tensor (ng,), as device tensors (owned by this
        object, overwritten by the next call)."""
        d = dens.contiguous()
        st = self._stream()
        _lib.check(_lib.lib.lres_lda_xc(self.s._ctx, d.data_ptr(), self.d_exc.data_ptr(), self.d_vxc.data_ptr(), st))
        _lib.check(_lib.lib.lres_hartree(self.s._ctx, d.data_ptr(), self.d_vh.data_ptr(), st))
        return self.d_exc, self.d_vxc, self.d_vh

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
             vion=None, step_times=None, device=None):
    """SCF to |n_out - n_in|_1 / N < tol (at most maxiter iterations).  device=None takes the
    device path when the solver offers density_device, the grid steps are this module's
    GridOps and a GPU is present.  Returns the dict of the reference's
    scf_lcao (energy, density, iterations, time, converged, dens_in, eband, ...)."""
    if device is None:
        device = (hasattr(solver, "density_device") and (grid is None or isinstance(grid, GridOps))
                  and torch.cuda.is_available())
    if device:
        return _scf_device(cr, solver, tol, maxiter, mix, ndiis, verbose, dens0, grid, vion, step_times)
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


def _diis_coefficients(gram):
    """Coefficients c (sum 1) minimising |sum c_i r_i| from the Gram matrix of the residuals:
    the bordered system [[G, 1], [1^T, 0]] [c, -lambda] = [0, 1], least squares (minimum norm,
    as numpy's lstsq) so that a singular G still gives an answer."""
    k = gram.shape[0]
    bm = np.zeros((k + 1, k + 1))
    bm[:k, :k] = gram
    bm[k, :k] = bm[:k, k] = 1.0
    rhs = np.zeros(k + 1)
    rhs[k] = 1.0
    return np.linalg.lstsq(bm, rhs, rcond=None)[0][:k]


def _scf_device(cr, solver, tol, maxiter, mix, ndiis, verbose, dens0, grid, vion, step_times):
    t0 = time.perf_counter()
    grid = GridOps(solver) if grid is None else grid
    dev = grid.dev
    if vion is None:
        vion_d = grid.ion_potential_device()
    else:
        vion_d = torch.as_tensor(np.ascontiguousarray(vion, dtype=np.float64).ravel(), device=dev)
    N, dV = float(cr.n_elec), float(cr.dV)
    if dens0 is None:
        dens = torch.full((cr.ng,), N / (cr.ng * dV), dtype=torch.float64, device=dev)
    else:
        dens = torch.as_tensor(np.ascontiguousarray(dens0, dtype=np.float64).ravel(), device=dev).clone()
    hist_n, hist_r = [], []
    converged = False
    nout = eband = None
    for it in range(1, maxiter + 1):
        ts = time.perf_counter()
        exc, vxc, vh = grid.lda_hartree_device(dens)
        v = vion_d + vh + vxc
        out = solver.density_device(v)
        nout, eband = out[0].reshape(-1), out[1]
        resid = nout - dens
        err = float(resid.abs().sum()) * dV / N           # the one scalar of the convergence test
        if verbose:
            print(f"  it {it:2d} |dn|/N = {err:.2e}  ({time.perf_counter() - ts:.2f}s)", flush=True)
        if err < tol:
            converged = True
            if step_times is not None:
                step_times.append(time.perf_counter() - ts)
            break
        hist_n.append(dens)
        hist_r.append(resid)
        if len(hist_n) > ndiis:
            hist_n.pop(0)
            hist_r.pop(0)
        k = len(hist_n)
        if k > 1:
            R = torch.stack(hist_r)
            coef = _diis_coefficients((R @ R.T).cpu().numpy())
            c = torch.as_tensor(coef, dtype=torch.float64, device=dev)
            dens = c @ torch.stack(hist_n) + mix * (c @ R)
        else:
            dens = dens + mix * resid
        dens = torch.clamp(dens, min=1e-12)
        dens = dens * ((N / dV) / dens.sum())
        if step_times is not None:
            torch.cuda.synchronize()
            step_times.append(time.perf_counter() - ts)
    exc, vxc, vh = grid.lda_hartree_device(dens)
    E_H = 0.5 * float(torch.dot(dens, vh)) * dV
    E_xc = float(torch.dot(dens, exc)) * dV
    E = eband - float(torch.dot(vh + vxc, dens)) * dV + E_H + E_xc
    sh = cr.shape
    return dict(energy=E, density=nout.cpu().numpy().reshape(sh), iterations=it, time=time.perf_counter() - t0,
                converged=converged, dens_in=dens.cpu().numpy().reshape(sh), eband=eband,
                last=(nout.cpu().numpy().reshape(sh), eband, out[2]), E_H=E_H, E_xc=E_xc)
