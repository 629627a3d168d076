"""Host-side system description: periodic crystal, H2 geometry generators and the
LCAO-on-grid basis that the window solve consumes.

This is one-time input preparation (the reference does it in numpy as well); the
per-iteration work on these inputs runs on the GPU.  Arithmetic follows the
reference operation by operation, so that the basis matrices (X, S, T) and
therefore the window problems are the reference's to the last bit or two:

* ``Crystal`` / ``h2_crystal``         lrft/three_d.py:41-87
* ``LCAOBasis``                         lrft/lcao3d.py:49-100
* ``cell_centres``                      lrft/lcao3d.py:287-289
* ``fd_hamiltonian`` (FD kinetic part)  lrft/three_d.py:151-164
* ``amorphous_h2`` (random sequential addition)  benchmarks/referee_checks.py:128-141

Two generators have no reference counterpart and follow the workload definitions
of the batched benchmark: ``cubic_h2`` (no jitter, bond along z) and
``jittered_h2`` (uniform centre jitter, isotropic random bond axes).
"""
from __future__ import annotations

import os
from dataclasses import dataclass

import numpy as np
from scipy import sparse

S_EXPS = (1.0, 0.3, 0.12)     # lrft/lcao3d.py:37
P_EXPS = (0.5,)               # lrft/lcao3d.py:38


@dataclass
class Crystal:
    """Periodic orthorhombic supercell sampled on a uniform grid (lrft/three_d.py:41-71)."""
    pos: np.ndarray           # (natoms, 3) bohr
    Z: np.ndarray             # (natoms,) ionic charges
    cell: np.ndarray          # (3,) box lengths
    shape: tuple              # grid points per axis
    rc: float = 1.0           # erf softening radius of the local pseudopotential
    rcs: np.ndarray = None
    charge: int = 0

    @property
    def atom_rc(self):
        return np.full(len(self.Z), self.rc) if self.rcs is None else np.asarray(self.rcs, float)

    @property
    def dx(self):
        return self.cell[0] / self.shape[0]

    @property
    def n_elec(self):
        return int(round(self.Z.sum())) - int(self.charge)

    @property
    def ng(self):
        return int(np.prod(self.shape))

    @property
    def dV(self):
        return float(np.prod(self.cell / np.array(self.shape)))


def _crystal(pos, n, a, pts_per_cell, rc):
    cell = a * np.array(n, float)
    shape = tuple(int(pts_per_cell * m) for m in n)
    return Crystal(np.array(pos), np.ones(len(pos)), cell, shape, rc)


def h2_crystal(n=(2, 2, 2), a=4.5, bond=1.4, pts_per_cell=8, jitter=0.15, seed=0, rc=1.0):
    """One H2 per cell, normal centre jitter, random axis (lrft/three_d.py:74-87)."""
    rng = np.random.default_rng(seed)
    pos = []
    for i in range(n[0]):
        for j in range(n[1]):
            for k in range(n[2]):
                c = (np.array([i, j, k]) + 0.5) * a + rng.normal(scale=jitter, size=3)
                u = rng.normal(size=3)
                u /= np.linalg.norm(u)
                pos += [c - 0.5 * bond * u, c + 0.5 * bond * u]
    return _crystal(pos, n, a, pts_per_cell, rc)


def cubic_h2(n=(3, 3, 3), a=4.5, bond=1.4, pts_per_cell=8, rc=1.0):
    """Simple-cubic H2 crystal: molecules at the cell centres, bonds along z, no jitter."""
    pos = []
    u = np.array([0.0, 0.0, 1.0])
    for i in range(n[0]):
        for j in range(n[1]):
            for k in range(n[2]):
                c = (np.array([i, j, k]) + 0.5) * a
                pos += [c - 0.5 * bond * u, c + 0.5 * bond * u]
    return _crystal(pos, n, a, pts_per_cell, rc)


def jittered_h2(n=(8, 8, 8), a=4.5, bond=1.4, pts_per_cell=8, jitter=0.1, seed=0, rc=1.0):
    """H2 crystal with centres displaced by U(-jitter, jitter) per axis and bond axes
    uniform on the sphere (normalised N(0, I3)); same loop order and generator as
    ``h2_crystal``."""
    rng = np.random.default_rng(seed)
    pos = []
    for i in range(n[0]):
        for j in range(n[1]):
            for k in range(n[2]):
                c = (np.array([i, j, k]) + 0.5) * a + rng.uniform(-jitter, jitter, size=3)
                u = rng.normal(size=3)
                u /= np.linalg.norm(u)
                pos += [c - 0.5 * bond * u, c + 0.5 * bond * u]
    return _crystal(pos, n, a, pts_per_cell, rc)


def min_image(d, L):
    """Minimum-image displacement (lrft/lcao3d.py:45-46)."""
    return d - L * np.round(d / L)


def amorphous_h2(nmol=512, box=36.0, dmin=3.0, bond=1.4, seed=7, shape=None, rc=1.0):
    """Random sequential addition of H2 centres with a minimum centre distance, random
    axes (benchmarks/referee_checks.py:128-141).  ``shape`` defaults to the
    reference's 0.6 bohr spacing; returns (crystal, centres)."""
    rng = np.random.default_rng(seed)
    centres = []
    L = np.full(3, box)
    while len(centres) < nmol:
        c = rng.uniform(0, box, 3)
        if centres:
            Q = np.array(centres)
            if np.min(np.linalg.norm(min_image(c - Q, L), axis=1)) < dmin:
                continue
        centres.append(c)
    pos = []
    for c in centres:
        u = rng.normal(size=3)
        u /= np.linalg.norm(u)
        pos += [c - 0.5 * bond * u, c + 0.5 * bond * u]
    if shape is None:
        m = int(round(box / 0.6))
        shape = (m, m, m)
    return Crystal(np.array(pos), np.ones(2 * nmol), np.full(3, float(box)), tuple(shape), rc), np.array(centres)


def cell_centres(n, a):
    """Centres of an n0 x n1 x n2 block of cubic cells (lrft/lcao3d.py:287-289)."""
    g = np.array([[i, j, k] for i in range(n[0]) for j in range(n[1]) for k in range(n[2])], float)
    return (g + 0.5) * a


def fd_hamiltonian(cr: Crystal, v):
    """Periodic 7-point finite-difference Hamiltonian -Lap/2 + v (lrft/three_d.py:151-164)."""
    dx = cr.dx
    idx = np.arange(cr.ng).reshape(cr.shape)
    rows, cols = [], []
    for ax in range(3):
        for s in (1, -1):
            rows.append(idx.ravel())
            cols.append(np.roll(idx, s, axis=ax).ravel())
    rows = np.concatenate(rows)
    cols = np.concatenate(cols)
    off = sparse.csr_matrix((np.full(rows.size, -0.5 / dx**2), (rows, cols)), shape=(cr.ng, cr.ng))
    return (off + sparse.diags(v.ravel() + 3.0 / dx**2)).tocsr()


class LCAOBasis:
    """s/p Gaussians times the compact cutoff (1-(r/rcut)^2)^2 tabulated on the grid,
    each normalised on the grid; S = X^T X dV and T = X^T T_FD X dV
    (lrft/lcao3d.py:49-96).  Functions of one atom are contiguous and share one
    support, which the GPU side uses to assemble H(v) by atom pairs.

    The tabulation is numpy, operation by operation as in the reference.  The sparse
    assembly (X from the tabulated points, X^T X, X^T T_FD X) runs in the native
    library (``assembly="native"``, lres_basis_build: the reference's scipy sums in
    their order, per atom pair, on the cores this process may use, or ``nthreads``);
    ``assembly="scipy"`` forms them with scipy.sparse as the reference does.
    ``tabulation="gpu"`` tabulates on the GPU instead (lres_basis_tabulate: the same points,
    values within a few ulp of numpy's exp and normalisation sums), then assembles natively."""

    def __init__(self, cr: Crystal, rcut=5.5, s_exps=None, p_exps=None, atom_exps=None, assembly="native",
                 nthreads=None, tabulation="numpy"):
        self.cr, self.rcut = cr, rcut
        s_exps = S_EXPS if s_exps is None else s_exps
        p_exps = P_EXPS if p_exps is None else p_exps
        if tabulation not in ("numpy", "gpu"):
            raise ValueError(f"tabulation must be 'numpy' or 'gpu', not {tabulation!r}")
        if tabulation == "gpu":
            if assembly != "native":
                raise ValueError("the GPU tabulation feeds the native assembly (assembly='native')")
            self._init_gpu(s_exps, p_exps, atom_exps, nthreads)
            return
        dx = cr.dx
        n1, n2, n3 = cr.shape
        rad = int(np.ceil(rcut / dx))
        off = np.arange(-rad, rad + 1)
        cube = np.stack(np.meshgrid(off, off, off, indexing="ij"), -1).reshape(-1, 3)
        if assembly == "native" and np.all((rad + 1) * dx < 0.5 * np.asarray(cr.cell, float)):
            # The cube stays inside half the cell, so the minimum image leaves every offset
            # as it is, and offsets more than rad + 1 points from the centre lie farther than
            # (rad + 1 - sqrt(3)/2) dx > rcut: the mask below would drop them.  Leaving them
            # out keeps the same points in the same order with the same values.
            cube = cube[np.sum(cube**2, axis=1) <= (rad + 1) ** 2]
        idxs, blocks, atom_of_fn, fn_ptr = [], [], [], [0]
        fn = 0
        for a, R in enumerate(cr.pos):
            if atom_exps is not None:
                s_exps, p_exps = atom_exps[a]
            c = np.round(R / dx).astype(int)
            P = c + cube
            d = P * dx - R
            d = min_image(d, cr.cell)
            r = np.linalg.norm(d, axis=1)
            m = r < rcut
            P, d, r = P[m], d[m], r[m]
            idx = np.ravel_multi_index((P[:, 0] % n1, P[:, 1] % n2, P[:, 2] % n3), cr.shape)
            cut = (1 - (r / rcut) ** 2) ** 2
            funcs = [np.exp(-al * r**2) * cut for al in s_exps]
            for al in p_exps:
                g = np.exp(-al * r**2) * cut
                funcs += [d[:, 0] * g, d[:, 1] * g, d[:, 2] * g]
            idxs.append(idx)
            blocks.append([f / np.sqrt(np.sum(f**2) * cr.dV) for f in funcs])
            atom_of_fn += [a] * len(funcs)
            fn += len(funcs)
            fn_ptr.append(fn)
        self.nb = fn
        self.atom_of_fn = np.array(atom_of_fn)
        self.atom_fn_ptr = np.array(fn_ptr, dtype=np.int64)   # functions of atom a: [ptr[a], ptr[a+1])
        if assembly == "native":
            self._assemble_native(idxs, blocks, nthreads)
        elif assembly == "scipy":
            rows = [idx for idx, blk in zip(idxs, blocks) for _ in blk]
            cols = [np.full(idx.size, f) for f, idx in enumerate(rows)]
            self.X = sparse.csc_matrix((np.concatenate([f for blk in blocks for f in blk]),
                                        (np.concatenate(rows), np.concatenate(cols))), shape=(cr.ng, fn))
            self.Xr = self.X.tocsr()
            self._matrices()
        else:
            raise ValueError(f"assembly must be 'native' or 'scipy', not {assembly!r}")

    def _init_gpu(self, s_exps, p_exps, atom_exps, nthreads):
        """The tabulation on the GPU (lres_basis_tabulate: same points, values within a
        few ulp of numpy's), then the native sparse assembly."""
        from . import _lib
        cr = self.cr
        nat = len(cr.pos)
        se = [atom_exps[a][0] if atom_exps is not None else s_exps for a in range(nat)]
        pe = [atom_exps[a][1] if atom_exps is not None else p_exps for a in range(nat)]
        cnt, idx, val = _lib.basis_tabulate(cr.pos, se, pe, cr.shape, cr.cell, cr.dx, self.rcut, cr.dV)
        nf = np.array([len(se[a]) + 3 * len(pe[a]) for a in range(nat)], np.int64)
        self.nb = int(nf.sum())
        self.atom_of_fn = np.repeat(np.arange(nat), nf)
        self.atom_fn_ptr = np.concatenate([[0], np.cumsum(nf)]).astype(np.int64)
        self._assemble_arrays(cnt, idx, val, nthreads)

    def _assemble_native(self, idxs, blocks, nthreads):
        cnt = np.array([idx.size for idx in idxs], np.int64)
        self._assemble_arrays(cnt, np.concatenate(idxs), np.concatenate([f for blk in blocks for f in blk]),
                              nthreads)

    def _assemble_arrays(self, cnt, idx, val, nthreads):
        from . import _lib
        cr = self.cr
        if nthreads is None:        # the cores this process may run on
            nthreads = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
        dx = cr.dx
        (Xp, Xi, Xv), (Rp, Ri, Rv), (Sp, Si, Sv), (Tp, Ti, Tv) = _lib.basis_matrices(
            self.atom_fn_ptr, cnt, idx, val, cr.shape, cr.dV, 3.0 / dx**2, -0.5 / dx**2, nthreads)
        ng, nb = cr.ng, self.nb
        self.X = sparse.csc_matrix((Xv, Xi, Xp), shape=(ng, nb))
        self.Xr = sparse.csr_matrix((Rv, Ri, Rp), shape=(ng, nb))
        self.S = sparse.csr_matrix((Sv, Si, Sp), shape=(nb, nb))
        self.T = sparse.csr_matrix((Tv, Ti, Tp), shape=(nb, nb))
        for A in (self.X, self.Xr, self.S, self.T):
            A.has_sorted_indices = True

    def _matrices(self):
        """S and T with scipy.sparse, as the reference forms them (lrft/lcao3d.py:86-96)."""
        dV = self.cr.dV
        self.S = (self.X.T @ self.X).tocsr() * dV
        T = fd_hamiltonian(self.cr, np.zeros(self.cr.shape))
        self.T = (self.X.T @ (T @ self.X)).tocsr() * dV

    def H(self, v):
        """Host reference of H(v) = T + X^T diag(v) X dV (lrft/lcao3d.py:98-100); the
        GPU solver assembles H on the device instead."""
        Xv = self.Xr.multiply(v.reshape(-1, 1)).tocsc()
        return (self.T + (self.X.T @ Xv) * self.cr.dV).tocsr()


def csr64(A):
    """Sorted CSR with int64 indices (lrft/lcao3d.py:297-300)."""
    A = A.tocsr()
    A.sort_indices()
    return (A.indptr.astype(np.int64), A.indices.astype(np.int64), np.ascontiguousarray(A.data, dtype=np.float64))
