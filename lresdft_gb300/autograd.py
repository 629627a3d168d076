"""torch.autograd Functions over the LRes band-energy adjoint (lres_adjoint).

``BandEnergy.apply(v, solver)`` is E_band at fixed electron number as a function of the
grid local potential v (a float64 CUDA tensor of the grid's shape): forward assembles
H(v) on the device and solves mu with e_lo fixed; backward returns grad * dE/dv.
``WindowBandEnergy.apply(HW, SW, solver)`` is the same energy as a function of the dense
window matrices (flat window layout, see ``LResGPU.window_offsets``) and returns
dE/dH_W and dE/dS_W.  The reference has no differentiable path; the derivative is the
closed form of the pole rule (dG = G dH G, dG = -z G dS G) with the fixed-N shift
kappa = (dE/dmu)/(dN/dmu).
"""
from __future__ import annotations

import numpy as np
import torch


def device_tensor(ptr, n):
    """A float64 CUDA tensor viewing n doubles at a device address (no copy)."""

    class _View:
        __cuda_array_interface__ = {"shape": (int(n),), "typestr": "<f8", "data": (int(ptr), False),
                                    "version": 3}
    return torch.as_tensor(_View(), device="cuda")


def window_matrices(solver):
    """Copies of the solver's current (H_W, S_W) as flat float64 CUDA tensors."""
    h, s = solver.window_ptrs()
    n = int(solver.window_offsets[-1])
    torch.cuda.synchronize()
    return device_tensor(h, n).clone(), device_tensor(s, n).clone()


def _ensure_state(solver, v=None):
    if solver.mu is None or solver.e_lo is None:
        if v is None:
            raise RuntimeError("the solver needs (mu, e_lo): call solver.density(v) once first")
        solver.density(v.detach().cpu().numpy().reshape(solver.b.cr.shape))


class BandEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, v, solver, tol=1e-10):
        v = v.detach().contiguous()
        _ensure_state(solver, v)
        torch.cuda.synchronize()
        solver.set_potential_device(v.data_ptr())
        mu, N, E = solver.solve_mu_fixed_n(tol=tol)
        solver.mu = mu
        ctx.solver, ctx.mu = solver, mu
        ctx.save_for_backward(v)
        return torch.tensor(E, dtype=torch.float64, device=v.device)

    @staticmethod
    def backward(ctx, g):
        (v,) = ctx.saved_tensors
        s = ctx.solver
        torch.cuda.synchronize()
        s.set_potential_device(v.data_ptr())
        dv = torch.empty_like(v)
        s.adjoint_device(ctx.mu, s.e_lo, dv_ptr=dv.data_ptr())
        return g * dv, None, None


class WindowBandEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, HW, SW, solver, tol=1e-10):
        HW, SW = HW.detach().contiguous(), SW.detach().contiguous()
        if solver.mu is None or solver.e_lo is None:
            raise RuntimeError("the solver needs (mu, e_lo): call solver.density(v) once first")
        torch.cuda.synchronize()
        solver.set_windows_device(HW.data_ptr(), SW.data_ptr())
        mu, N, E = solver.solve_mu_fixed_n(tol=tol)
        solver.mu = mu
        ctx.solver, ctx.mu = solver, mu
        ctx.save_for_backward(HW, SW)
        return torch.tensor(E, dtype=torch.float64, device=HW.device)

    @staticmethod
    def backward(ctx, g):
        HW, SW = ctx.saved_tensors
        s = ctx.solver
        torch.cuda.synchronize()
        s.set_windows_device(HW.data_ptr(), SW.data_ptr())
        dH, dS = torch.empty_like(HW), torch.empty_like(SW)
        s.adjoint_device(ctx.mu, s.e_lo, dHW_ptr=dH.data_ptr(), dSW_ptr=dS.data_ptr())
        return g * dH, g * dS, None, None
