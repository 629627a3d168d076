"""Drop-in GPU replacement of the reference's LRes window solver.

``LResGPU`` has the constructor, attributes and ``density(v, N=None) -> (dens,
e_band, mu)`` protocol of ``LRFTLCAOCpp`` (lrft/lcao3d.py:340-456), so that
``scf_lcao``, the command-line front end (``make_solvers``, lrft/cli.py:150-170) and
the benchmarks take it unchanged.  It evaluates the window density by the pole
route on the GPU (one fused launch for all windows x M/2 poles, liblres_gb300)
instead of per-window eigendecompositions; the mu logic keeps the reference's
warm/cold decisions:

* warm step (lrft/lcao3d.py:413-448): keep mu and e_lo if the smallest window
  eigenvalue lies in (e_lo + margin/3, e_lo + 2 margin) and below the truncation
  edge c + 1.5 R; the reference reads it from its window spectra, here two
  Sylvester-inertia counts decide it; keep mu if |N(mu) - N| <= 1e-8 N (1e-7 N in
  mixed precision, the FP32 count-noise floor), else solve for mu and return the
  density of a pass at the new mu (the reference with reuse_vectors=False; the pole
  route stores no eigenvectors, so reuse_vectors is accepted for signature
  compatibility only);
* cold step (lrft/lcao3d.py:449-456): e_lo = lambda_min - margin with lambda_min
  from inertia bisection; mu bracketed from the previous accepted mu when there is one
  (the count is monotone in mu, so the root is the same), else from
  [max(lambda_min, e_lo+1e-6), +1] widened by 0.5 (lrft/lcao3d.py:387-398).

Each N(mu) evaluation is a pole pass (the poles move with mu), so mu is found by
Brent's method on pass results; the last pass at the accepted mu is the density.  On
the default tridiagonal route (liblres_gb300, LRES_ROUTE_TRIDIAG) every window's
standard form is reduced once per Hamiltonian to tridiagonal form, so each pass costs
O(M/2 x rows x n_W) instead of M/2 dense factorisations; the inertia counts of the mu
logic are then Sturm counts of those tridiagonal matrices.
With trace rows installed (fine grids) the trial passes run over them and produce no
density; the accepted mu then gets one density pass over the owned points.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from .system import csr64, min_image


class StaleMu(RuntimeError):
    """The warm-start mu was too far off (lrft/lcao3d.py:41-42)."""


def window_setup(basis, cells, R_w):
    """Windows W(B) and owned grid points own(B) of lrft/lcao3d.py:135-160; the
    Voronoi ownership runs on the GPU with the reference's operation order."""
    cr = basis.cr
    d = min_image(cr.pos[:, None, :] - cells[None, :, :], cr.cell)
    cell_of_atom = np.argmin(np.linalg.norm(d, axis=2), axis=1)
    cell_of_fn = cell_of_atom[np.asarray(basis.atom_of_fn)]
    dc = np.linalg.norm(min_image(cells[:, None, :] - cells[None, :, :], cr.cell), axis=2)
    owner = _lib.voronoi_owner(cr.shape, cr.cell, cells)
    windows = [np.where(np.isin(cell_of_fn, np.where(dc[B] <= R_w)[0]))[0] for B in range(len(cells))]
    order = np.argsort(owner, kind="stable")
    counts = np.bincount(owner, minlength=len(cells))
    offs = np.concatenate([[0], np.cumsum(counts)])
    own = [order[offs[B]:offs[B + 1]] for B in range(len(cells))]
    return windows, own, owner


def _groups(basis):
    """Function ranges of the atoms: functions of an atom are contiguous (lrft/lcao3d.py:61-84)."""
    aof = np.asarray(basis.atom_of_fn)
    if aof.size and np.any(np.diff(aof) < 0):
        raise ValueError("basis functions of one atom must be contiguous")
    natoms = int(aof.max()) + 1 if aof.size else 0
    counts = np.bincount(aof, minlength=natoms)
    return np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)


def _plain_lcao(basis):
    """True if basis.H(v) is T + X^T diag(v) X dV, which the GPU assembles itself."""
    H = getattr(type(basis), "H", None)
    return (H is not None and getattr(H, "__qualname__", "") == "LCAOBasis.H" and hasattr(basis, "T")
            and hasattr(basis, "Xr"))


def solved_windows(basis, windows, own, merge=True):
    """The windows the GPU solves, from the reference's windows and ownership:

    * windows with identical function sets (R_w reaching across the cell) merged into one
      with the union of their owned points (N, E_band and the density are sums over owned
      points of the same resolvent);
    * within each, the atoms whose functions vanish on every owned point first (whole atoms,
      each group in its original order): the owned-point rows are then zero in those leading
      columns and the pole kernel starts them at the first column an owned point touches.

    Returns (windows, owned points, index of the solved window of every input window)."""
    cw, cown = list(windows), list(own)
    ctx_of = np.arange(len(windows))
    if merge:
        first, groups = {}, []
        for B, W in enumerate(windows):
            key = np.asarray(W).tobytes()
            if key not in first:
                first[key] = len(groups)
                groups.append([])
            groups[first[key]].append(B)
        if len(groups) < len(windows):
            for k, gr in enumerate(groups):
                ctx_of[gr] = k
            cw = [windows[gr[0]] for gr in groups]
            cown = [np.sort(np.concatenate([own[B] for B in gr])) for gr in groups]
    aof = np.asarray(basis.atom_of_fn)
    ordered = []
    for W, o in zip(cw, cown):
        sub = basis.Xr[o]
        touched = np.zeros(int(aof.max()) + 1, bool)
        touched[aof[sub.indices[sub.data != 0]]] = True
        t = touched[aof[W]]
        ordered.append(np.concatenate([W[~t], W[t]]) if t.any() and not t.all() else W)
    return ordered, cown, ctx_of


def trace_factor(K, rtol=1e-14):
    """R with R^T R = K for a window's owned-row Gram matrix K = F^T F, built on the block
    from the first column with a nonzero diagonal on (the columns before it are exactly zero
    in R, as they are in F).

    Pivoted Cholesky (LAPACK pstrf), stopped when every remaining pivot is below rtol times
    the largest diagonal entry: K[p][:, p] = U^T U, R = U with its columns put back in place.
    Rank-revealing like an eigendecomposition (at most rank(K) rows) at a tenth of the cost.
    The eigendecomposition Lambda^1/2 V^T (eigenvalues above rtol * max) is the fallback."""
    n = K.shape[0]
    nz = np.flatnonzero(np.diag(K) > 0)
    c0 = int(nz[0]) if nz.size else n
    Ks = np.array(K[c0:, c0:], dtype=np.float64, order="F")
    top = float(np.max(np.diag(Ks))) if Ks.size else 0.0
    if top <= 0:
        return np.zeros((0, n))
    from scipy.linalg import lapack
    pstrf = getattr(lapack, "dpstrf", None)
    if pstrf is not None:
        try:
            U, piv, rank, info = pstrf(Ks, tol=rtol * top, lower=0)
        except (TypeError, ValueError):       # a scipy whose wrapper differs: use the fallback
            info = -1
        if info >= 0:
            R = np.zeros((int(rank), n))
            R[:, c0 + piv - 1] = np.triu(U)[:rank]
            return R
    lam, V = np.linalg.eigh(Ks)
    keep = lam > rtol * lam[-1]
    R = np.zeros((int(keep.sum()), n))
    R[:, c0:] = np.sqrt(lam[keep])[:, None] * V[:, keep].T
    return R


class LResGPU:
    """GPU pole-route LRes window solver with the LRFTLCAOCpp interface.

    Extra keywords: ``precision`` "fp64" (complex128 factor/solve throughout) or
    "mixed" (complex64 factor/solve of the standard-form windows
    L^-1 (z S - H) L^-T, FP64 Cholesky/orthogonalisation, FP64 pole sums, electron
    count and energies); ``route`` "auto" (the library's choice: tridiagonal unless the
    context has fewer than 4 windows or windows too large for it), "tridiag" or "ldl"
    (one dense LDL^T per window and pole)."""

    def __init__(self, basis, cells, R_w=12.1, M=64, margin=0.3, nthreads=1, lag_mu=False, reuse_vectors=True,
                 precision="fp64", tile_config=None, trace_rows="auto", merge_windows="auto", route="auto"):
        if M % 2 or M < 2:
            raise ValueError(f"M must be even and >= 2 (got {M})")
        if precision not in ("fp64", "mixed"):
            raise ValueError(f"precision must be 'fp64' or 'mixed' (got {precision!r})")
        if not R_w > 0:
            raise ValueError(f"R_w must be positive (got {R_w})")
        if not (tile_config is None or tile_config == "auto" or tile_config in range(6)):
            raise ValueError(f"tile_config must be None, 'auto' or 0..5 (got {tile_config!r})")
        if route not in ("auto", "tridiag", "ldl"):
            raise ValueError(f"route must be 'auto', 'tridiag' or 'ldl' (got {route!r})")
        self.b, self.M, self.margin = basis, M, margin
        self.lag_mu, self.reuse_vectors, self.nthreads = lag_mu, reuse_vectors, nthreads
        self.precision = precision
        cr = basis.cr
        cells = np.asarray(cells, float)
        self.windows, self.own, self.owner = window_setup(basis, cells, R_w)
        self.nW = np.array([len(W) for W in self.windows])
        self.Wflat = np.concatenate(self.windows).astype(np.int64)
        self.Woff = np.concatenate([[0], np.cumsum(self.nW)]).astype(np.int64)
        self.Oflat = np.concatenate(self.own).astype(np.int64)
        self.Ooff = np.concatenate([[0], np.cumsum([len(o) for o in self.own])]).astype(np.int64)
        # the windows the GPU solves (merged identical windows, atoms reordered)
        cw, cown, self._ctx_of = solved_windows(basis, self.windows, self.own, merge=bool(merge_windows))
        self.ctx_windows, self.ctx_own = cw, cown
        self.ctx_nW = np.array([len(W) for W in cw])
        cWflat = np.concatenate(cw).astype(np.int64)
        cWoff = np.concatenate([[0], np.cumsum(self.ctx_nW)]).astype(np.int64)
        cOflat = np.concatenate(cown).astype(np.int64)
        cOoff = np.concatenate([[0], np.cumsum([len(o) for o in cown])]).astype(np.int64)
        self.gptr = _groups(basis)
        self.mu = self.e_lo = None
        self.passes = 0
        self.inertia_calls = 0
        self._slope = None
        self._mu_last = None       # last accepted mu (survives StaleMu / cold steps)
        self._lam_min = None       # last smallest window eigenvalue
        self.trace = None          # set to a list to record (mu, N(mu)) of every pass
        self._gpu_h = _plain_lcao(basis)
        X, S = csr64(basis.Xr), csr64(basis.S)
        T = csr64(basis.T) if hasattr(basis, "T") else None
        d = _lib.SystemDesc()
        d.nb = basis.nb
        d.shape[:] = [int(s) for s in cr.shape]
        d.cell[:] = [float(x) for x in cr.cell]
        d.dV = cr.dV
        d.Xp, d.Xi, d.Xv = _lib.ptr64(X[0]), _lib.ptr64(X[1]), _lib.ptrd(X[2])
        d.Sp, d.Si, d.Sv = _lib.ptr64(S[0]), _lib.ptr64(S[1]), _lib.ptrd(S[2])
        if T is not None:
            d.Tp, d.Ti, d.Tv = _lib.ptr64(T[0]), _lib.ptr64(T[1]), _lib.ptrd(T[2])
        d.ngroups = len(self.gptr) - 1
        d.gptr = _lib.ptr64(self.gptr)
        d.nwin = len(cw)
        d.Wflat, d.Woff = _lib.ptr64(cWflat), _lib.ptr64(cWoff)
        d.Oflat, d.Ooff = _lib.ptr64(cOflat), _lib.ptr64(cOoff)
        ctx = C.c_void_p()
        prec = {"fp64": _lib.LRES_FP64, "mixed": _lib.LRES_MIXED}[precision]
        _lib.check(_lib.lib.lres_ctx_create(C.byref(ctx), C.byref(d), prec, M, None))
        self._ctx = ctx
        self._keep = (X, S, T, cWflat, cWoff, cOflat, cOoff)   # referenced by the descriptor
        if route != "auto":
            self.set_route(route)
        # tile configuration of the pole kernel: an index, or "auto" to time all of them on
        # the first Hamiltonian (see autotune); None keeps the library default
        self.tile_config = tile_config
        # tile configurations: of the LDL^T kernel on that route, of the reduction and row panels
        # on the tridiagonal route; "auto" times them on the first Hamiltonian
        self._tuned = not (tile_config == "auto")
        if isinstance(tile_config, int):
            self.autotune(0.0, -1.0, config=tile_config)
        self._out = np.zeros(3)
        self.dens_buf = np.zeros(cr.ng)
        self._device_out = False
        self._v_keep = None
        # trace rows (passes that need N and E only): installed when the owned points
        # outnumber the window functions clearly (fine grids)
        self._trace = False
        self._resolved = False      # the last density call re-solved mu
        self.trace_rows = None
        m_w = np.diff(cOoff)
        if trace_rows is True or (trace_rows == "auto" and m_w.mean() > 1.5 * self.ctx_nW.mean()):
            self.install_trace_rows()

    def close(self):
        if getattr(self, "_ctx", None):
            _lib.lib.lres_ctx_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------------ GPU calls
    @property
    def route(self):
        """Route of the pole solves: "tridiag" or "ldl"."""
        r = C.c_int32()
        _lib.check(_lib.lib.lres_get_route(self._ctx, C.byref(r)))
        return "tridiag" if r.value == _lib.LRES_ROUTE_TRIDIAG else "ldl"

    @property
    def standard_form(self):
        """Kernel of the mixed tridiagonal route's FP32 standard form: "simt" or "tensor"."""
        r = C.c_int32()
        _lib.check(_lib.lib.lres_get_standard_form_kernel(self._ctx, C.byref(r)))
        return "tensor" if r.value == _lib.LRES_SF_TENSOR else "simt"

    def set_standard_form(self, kind):
        """Run the FP32 standard form on the SIMT pipes ("simt") or the tensor cores
        ("tensor"); takes effect at the next Hamiltonian."""
        code = {"simt": _lib.LRES_SF_SIMT, "tensor": _lib.LRES_SF_TENSOR}[kind]
        _lib.check(_lib.lib.lres_set_standard_form_kernel(self._ctx, code))

    def set_route(self, route):
        """Switch the route of the pole solves ("tridiag" or "ldl")."""
        code = {"tridiag": _lib.LRES_ROUTE_TRIDIAG, "ldl": _lib.LRES_ROUTE_LDL}[route]
        _lib.check(_lib.lib.lres_set_route(self._ctx, code, None))

    def set_potential(self, v):
        """H(v) for all windows: assembled on the GPU from v (a host array or a CUDA tensor of
        ng float64), or (for bases with extra terms in H) built by basis.H on the host and
        gathered on the GPU."""
        if hasattr(v, "is_cuda") and v.is_cuda:
            if self._gpu_h:
                import torch
                vd = v.detach().reshape(-1).to(torch.float64).contiguous()
                self._v_keep = vd                     # alive until the kernels have read it
                self.set_potential_device(vd.data_ptr(), torch.cuda.current_stream().cuda_stream)
                return
            v = v.detach().cpu().numpy()
        if self._gpu_h:
            v = _lib.f64(v).ravel()
            _lib.check(_lib.lib.lres_set_potential(self._ctx, v.ctypes.data, 0, None))
        else:
            self.set_hamiltonian(self.b.H(v))

    def set_potential_device(self, v_ptr, stream=None):
        """H(v) from a device array of ng doubles (stream-ordered, no host copy; capturable)."""
        _lib.check(_lib.lib.lres_set_potential(self._ctx, v_ptr, 1, stream))

    def pole_pass_device(self, mu, e_lo, dens_ptr=None):
        """Pole pass leaving the density on the device (copied to dens_ptr if given);
        returns (N(mu), E_band)."""
        self.passes += 1
        _lib.check(_lib.lib.lres_pass(self._ctx, float(mu), float(e_lo), dens_ptr, 1, _lib.ptrd(self._out), None))
        return float(self._out[0]), float(self._out[1])

    def pass_async(self, mu, e_lo, d_out_ptr, stream=None):
        """Capturable pass: no host synchronisation; N, E_band land in d_out_ptr[0..1]."""
        self.passes += 1
        _lib.check(_lib.lib.lres_pass_async(self._ctx, float(mu), float(e_lo), d_out_ptr, stream))

    def status(self):
        st = C.c_int32()
        _lib.check(_lib.lib.lres_status(self._ctx, C.byref(st), None))
        return int(st.value)

    def density_device_ptr(self):
        p = C.c_void_p()
        _lib.check(_lib.lib.lres_density_ptr(self._ctx, C.byref(p)))
        return p.value

    # ------------------------------------------------------------------ adjoint
    @property
    def window_offsets(self):
        """Offsets of each window's column-major n_W x n_W block in the flat window layout
        of set_windows / adjoint: the windows the GPU solves (``ctx_windows``, which are
        ``windows`` unless identical windows were merged)."""
        return np.concatenate([[0], np.cumsum(self.ctx_nW.astype(np.int64) ** 2)])

    def window_blocks(self, flat):
        """Per-window n_W x n_W matrices of a flat window-layout array (views)."""
        off = self.window_offsets
        return [flat[off[w]:off[w + 1]].reshape(n, n, order="F") for w, n in enumerate(self.ctx_nW)]

    def flatten_windows(self, mats):
        """Flat window-layout array of per-window matrices."""
        return np.concatenate([np.asarray(a, np.float64).ravel(order="F") for a in mats])

    def set_windows(self, HW=None, SW=None):
        """Replace the dense window matrices (flat window layout, host arrays); None keeps one."""
        h = None if HW is None else _lib.f64(HW)
        sw = None if SW is None else _lib.f64(SW)
        _lib.check(_lib.lib.lres_set_windows(self._ctx, None if h is None else h.ctypes.data,
                                             None if sw is None else sw.ctypes.data, 0, None))

    def window_ptrs(self):
        """Device addresses of the context's H_W and S_W arrays (flat window layout)."""
        h, sw = C.c_void_p(), C.c_void_p()
        _lib.check(_lib.lib.lres_window_ptrs(self._ctx, C.byref(h), C.byref(sw)))
        return h.value, sw.value

    def set_windows_device(self, HW_ptr=None, SW_ptr=None, stream=None):
        _lib.check(_lib.lib.lres_set_windows(self._ctx, HW_ptr, SW_ptr, 1, stream))

    def adjoint(self, mu=None, e_lo=None, windows=False):
        """Gradient of the band energy at fixed N (e_lo fixed) at (mu, e_lo), by default the
        state of the last density call, on the current Hamiltonian.  Returns a dict with
        N, E, dN/dmu, dE/dmu, kappa, dv (grid shape) and, with windows=True, the flat
        window-layout arrays dHW and dSW."""
        mu = self.mu if mu is None else mu
        e_lo = self.e_lo if e_lo is None else e_lo
        if mu is None or e_lo is None:
            raise RuntimeError("adjoint needs (mu, e_lo): call density() first or pass them")
        cr = self.b.cr
        dv = np.empty(cr.ng)
        size = int(self.window_offsets[-1])
        dHW = np.empty(size) if windows else None
        dSW = np.empty(size) if windows else None
        out = np.zeros(6)
        _lib.check(_lib.lib.lres_adjoint(self._ctx, float(mu), float(e_lo), dv.ctypes.data, 0,
                                         None if dHW is None else dHW.ctypes.data,
                                         None if dSW is None else dSW.ctypes.data, 0, _lib.ptrd(out), None))
        res = {"N": out[0], "E": out[1], "dNdmu": out[2], "dEdmu": out[3], "kappa": out[4],
               "dv": dv.reshape(cr.shape), "mu": float(mu), "e_lo": float(e_lo)}
        if windows:
            res["dHW"], res["dSW"] = dHW, dSW
        return res

    def adjoint_device(self, mu, e_lo, dv_ptr=None, dHW_ptr=None, dSW_ptr=None, stream=None):
        """lres_adjoint into device arrays; returns (N, E, dN/dmu, dE/dmu, kappa)."""
        out = np.zeros(6)
        _lib.check(_lib.lib.lres_adjoint(self._ctx, float(mu), float(e_lo), dv_ptr, 1, dHW_ptr, dSW_ptr, 1,
                                         _lib.ptrd(out), stream))
        return tuple(float(x) for x in out[:5])

    def owned_gram(self):
        """K_W = F_W^T F_W of every window (flat window layout), F_W = X[own(B), W]."""
        K = np.empty(int(self.window_offsets[-1]))
        _lib.check(_lib.lib.lres_owned_gram(self._ctx, K.ctypes.data, 0, None))
        return K

    def install_trace_rows(self, rtol=1e-14):
        """Factor R_W = Lambda^1/2 V^T of K_W = V Lambda V^T (eigenvalues above rtol * max kept)
        for every window and install it as the trace rows: passes without a density and the
        adjoint then run over r_W <= n_W rows instead of |own(B)|."""
        K = self.owned_gram()
        rows, blocks = [], []
        for Kw in self.window_blocks(K):
            R = trace_factor(Kw, rtol)
            rows.append(R.shape[0])
            blocks.append(R.ravel(order="F"))
        r_w = np.asarray(rows, np.int32)
        flat = np.ascontiguousarray(np.concatenate(blocks))
        _lib.check(_lib.lib.lres_set_trace_rows(self._ctx, r_w.ctypes.data, flat.ctypes.data, None))
        self._trace = True
        self.trace_rows = r_w

    def remove_trace_rows(self):
        _lib.check(_lib.lib.lres_set_trace_rows(self._ctx, None, None, None))
        self._trace = False
        self.trace_rows = None

    def solve_mu_fixed_n(self, N=None, mu0=None, tol=1e-10, maxiter=60):
        """mu with |N(mu) - N| <= tol (absolute) on the current Hamiltonian, e_lo fixed: a
        bracket grown from mu0 (default: the current mu) by steps of the stored slope, then
        Brent's method, on passes without density.  Returns (mu, N(mu), E_band(mu))."""
        N = self.b.cr.n_elec if N is None else N
        mu = self.mu if mu0 is None else mu0
        if mu is None or self.e_lo is None:
            raise RuntimeError("solve_mu_fixed_n needs (mu, e_lo): call density() first or set them")
        lo_bound = self.e_lo + 1e-6
        mu = max(mu, lo_bound + 1e-6)
        cache = {}

        def f(x):
            _, n, e = self.pole_pass(x, self.e_lo, want_density=False)
            cache[x] = (n, e)
            return n - N

        f0 = f(mu)
        if abs(f0) <= tol:
            return mu, cache[mu][0], cache[mu][1]
        slope = self._slope if self._slope and self._slope > 0 else max(N, 1.0)
        step = min(max(abs(f0) / slope, 1e-6), 0.1)
        a, fa = mu, f0
        for _ in range(maxiter):
            x = a - step if fa > 0 else a + step
            if x <= lo_bound:
                x = 0.5 * (a + lo_bound)
            fx = f(x)
            if abs(fx) <= tol:
                return x, cache[x][0], cache[x][1]
            if (fx > 0) != (fa > 0):
                b, fb = x, fx
                break
            a, fa = x, fx
            step *= 2.0
        else:
            raise RuntimeError("solve_mu_fixed_n: no sign change of N(mu) - N")
        x = self._brent(f, a, fa, b, fb, tol, xtol=1e-15, maxit=maxiter)
        return x, cache[x][0], cache[x][1]

    def set_hamiltonian(self, H):
        Hp, Hi, Hv = csr64(H)
        _lib.check(_lib.lib.lres_set_hamiltonian_csr(self._ctx, _lib.ptr64(Hp), _lib.ptr64(Hi), _lib.ptrd(Hv), None))

    def pole_pass(self, mu, e_lo, want_density=True):
        """One pole pass: returns (density or None, N(mu), E_band); the density is a host
        array, or a CUDA tensor while a density_device call runs."""
        self.passes += 1
        if want_density and self._device_out:
            import torch
            dens = torch.empty(self.b.cr.ng, dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()               # the device copy below runs on the legacy stream
            _lib.check(_lib.lib.lres_pass(self._ctx, float(mu), float(e_lo), dens.data_ptr(), 1,
                                          _lib.ptrd(self._out), None))
        else:
            dens = self.dens_buf if want_density else None
            ptr = dens.ctypes.data if want_density else None
            _lib.check(_lib.lib.lres_pass(self._ctx, float(mu), float(e_lo), ptr, 0, _lib.ptrd(self._out), None))
            dens = dens.copy() if want_density else None
        if self.trace is not None:
            self.trace.append((float(mu), float(self._out[0])))
        return dens, float(self._out[0]), float(self._out[1])

    def autotune(self, mu, e_lo, config=-1):
        """Pick the tile configuration of the route (-1: time all six on the current
        Hamiltonian and keep the fastest; on the LDL^T route with full passes at (mu, e_lo)).
        Returns (chosen, ms per config)."""
        chosen = C.c_int32()
        ms = np.full(6, -1.0)
        _lib.check(_lib.lib.lres_autotune(self._ctx, float(mu), float(e_lo), int(config), C.byref(chosen),
                                          _lib.ptrd(ms), None))
        return int(chosen.value), ms

    def timings(self):
        """Device milliseconds of the last launches: pole kernel, pole sums, H(v)
        assembly, window gather, standard-form transform, inertia kernel, tridiagonal
        reduction, rows through its reflectors (-1 = none)."""
        ms = np.empty(8)
        _lib.check(_lib.lib.lres_timings(self._ctx, _lib.ptrd(ms), 8))
        return dict(zip(("pole_kernel", "pole_sums", "assemble_h", "gather", "transform", "inertia",
                         "tri_reduce", "tri_rows"), ms))

    def window_sums(self):
        nw = np.empty(len(self.ctx_windows))
        ew = np.empty(len(self.ctx_windows))
        _lib.check(_lib.lib.lres_window_sums(self._ctx, _lib.ptrd(nw), _lib.ptrd(ew)))
        return nw, ew

    def inertia(self, sigma, per_window=False):
        """Number of window eigenvalues below sigma (total, or per window)."""
        self.inertia_calls += 1
        tot = C.c_int64()
        below = np.empty(len(self.ctx_windows), np.int32) if per_window else None
        bp = below.ctypes.data_as(C.POINTER(C.c_int32)) if per_window else None
        _lib.check(_lib.lib.lres_inertia(self._ctx, float(sigma), bp, C.byref(tot), None))
        # per window of ``windows`` (merged windows share their count); the total counts
        # each solved window once
        return below[self._ctx_of] if per_window else int(tot.value)

    def min_eig(self, lo, hi, tol=1e-12):
        out = C.c_double()
        _lib.check(_lib.lib.lres_min_eig(self._ctx, float(lo), float(hi), float(tol), C.byref(out), None))
        return float(out.value)

    # ------------------------------------------------------------------ mu logic
    def _upper(self, mu, e_lo):
        c, R = 0.5 * (mu + e_lo), 0.5 * (mu - e_lo)
        return c + 1.5 * R

    def _edge_ok(self, mu, e_lo):
        """lrft/lcao3d.py:420: some window state below c + 1.5 R and
        e_lo + margin/3 < lambda_min < e_lo + 2 margin."""
        if self.inertia(e_lo + self.margin / 3) > 0:
            return False
        return self.inertia(min(e_lo + 2 * self.margin, self._upper(mu, e_lo))) > 0

    def _solve_mu(self, e_lo, N, ftol, start=None, lo_start=None):
        """Root of N(mu) - N by Brent's method on pole passes.  `start` = (mu, f, dens,
        eb) of a pass already done (warm step: a secant step with the slope of the last
        solve, then widening secant steps until the count changes sign).  Returns
        (mu, dens, e_band) of the accepted pass."""
        cache = {}
        hist = []

        def f(x):
            dens, n, eb = self.pole_pass(x, e_lo, want_density=not self._trace)
            cache[x] = (dens, eb)
            hist.append((x, n - N))
            return n - N

        lo_bound = e_lo + 1e-6
        if start is not None:
            x0, f0, d0, e0 = start
            cache[x0] = (d0, e0)
            hist.append((x0, f0))
            # Newton step with the slope dN/dmu of the previous solve (at most 1 Ha, the width
            # of the reference's first bracket); stop if it lands within the tolerance, bracket
            # on a sign change, else continue with secant steps
            slope = self._slope if self._slope and self._slope > 0 else max(N, 1.0)
            step = -f0 / slope
            step = math.copysign(min(max(abs(step), 1e-7), 1.0), step)
            a, fa = x0, f0
            b = None
            for _ in range(40):
                x1 = a + step
                if x1 <= lo_bound:
                    x1 = 0.5 * (a + lo_bound)
                f1 = f(x1)
                if abs(f1) <= ftol:
                    self._note_slope(hist, x1)
                    return x1, cache[x1][0], cache[x1][1]
                if (f1 > 0) != (fa > 0):
                    b, fb = x1, f1
                    break
                # secant extrapolation from the last two points, 10% past its root so that the
                # next point brackets (twice the step where the count did not move)
                sec = -f1 * (x1 - a) / (f1 - fa) if f1 != fa else 2 * step
                step = math.copysign(min(abs(sec) * 1.1, 1.0), step)
                a, fa = x1, f1
            if b is None:
                raise StaleMu("no sign change of the electron count near the warm-start mu")
        else:
            lo = lo_start
            flo = f(lo)
            if flo > 0:
                raise RuntimeError("electron count positive at the bottom of the spectrum")
            hi = lo + 1.0
            fhi = f(hi)
            n_expand = 0
            while fhi < 0:
                hi += 0.5
                n_expand += 1
                if n_expand > 40:
                    raise StaleMu("window spectra hold fewer than N electrons")
                fhi = f(hi)
            a, fa, b, fb = lo, flo, hi, fhi
        x = self._brent(f, a, fa, b, fb, ftol, xtol=getattr(self, "_xtol", 1e-12))
        self._note_slope(hist, x)
        dens, eb = cache[x]
        return x, dens, eb

    def _note_slope(self, hist, x):
        """Local slope dN/dmu at the accepted root for the next warm start: the secant of
        the closest evaluations on both sides (or the two closest ones)."""
        below = [h for h in hist if h[1] < 0]
        above = [h for h in hist if h[1] > 0]
        if below and above:
            lb = min(below, key=lambda h: abs(h[0] - x))
            ub = min(above, key=lambda h: abs(h[0] - x))
        elif len(hist) >= 2:
            lb, ub = sorted(hist, key=lambda h: abs(h[0] - x))[:2]
        else:
            return
        if ub[0] != lb[0]:
            sl = (ub[1] - lb[1]) / (ub[0] - lb[0])
            if sl > 0:
                self._slope = sl

    @staticmethod
    def _brent(f, a, fa, b, fb, ftol, xtol=1e-12, maxit=100):
        """Brent's root finder (zeroin) on a bracket with fa*fb <= 0; stops when |f| <=
        ftol or the bracket is below xtol; returns an evaluated point."""
        if abs(fa) < abs(fb):
            a, fa, b, fb = b, fb, a, fa
        if abs(fb) <= ftol:
            return b
        c, fc = a, fa
        d = e = b - a
        for _ in range(maxit):
            if (fb > 0) == (fc > 0):
                c, fc = a, fa
                d = e = b - a
            if abs(fc) < abs(fb):
                a, b, c = b, c, b
                fa, fb, fc = fb, fc, fb
            tol1 = 2.0 * 2.2e-16 * abs(b) + 0.5 * xtol
            xm = 0.5 * (c - b)
            if abs(fb) <= ftol or abs(xm) <= tol1:
                return b
            if abs(e) >= tol1 and abs(fa) > abs(fb):
                s = fb / fa
                if a == c:
                    p, q = 2.0 * xm * s, 1.0 - s
                else:
                    q, r = fa / fc, fb / fc
                    p = s * (2.0 * xm * q * (q - r) - (b - a) * (r - 1.0))
                    q = (q - 1.0) * (r - 1.0) * (s - 1.0)
                if p > 0:
                    q = -q
                p = abs(p)
                if 2.0 * p < min(3.0 * xm * q - abs(tol1 * q), abs(e * q)):
                    e, d = d, p / q
                else:
                    d = e = xm
            else:
                d = e = xm
            a, fa = b, fb
            b = b + (d if abs(d) > tol1 else math.copysign(tol1, xm))
            fb = f(b)
        return b

    # ------------------------------------------------------------------ protocol
    def density_device(self, v, N=None):
        """density() with device tensors: v a CUDA tensor of ng float64 values, the returned
        density a CUDA tensor of the grid's shape (the same protocol and passes)."""
        self._device_out = True
        try:
            return self.density(v, N)
        finally:
            self._device_out = False

    def density(self, v, N=None):
        try:
            return self._density(v, N)
        except StaleMu:
            self.mu = None
            return self._density(v, N)

    def _density(self, v, N=None):
        cr = self.b.cr
        N = cr.n_elec if N is None else N
        self.set_potential(v)
        if not self._tuned:
            # time the tile configurations once, on this Hamiltonian, at a mu near the gap
            lm = self.min_eig(-1.0, 0.0, tol=1e-6)
            self.tile_config, self.tune_ms = self.autotune(lm + 0.4, lm - 0.3)
            self._tuned = True
        # count tolerances: the reference's 1e-8 N (lrft/lcao3d.py:412) for the FP64 path
        # and a root tolerance far below it; the complex64 path's counts carry ~1e-7 N of
        # FP32 noise, so both tolerances sit at that floor
        if self.precision == "fp64":
            tol, ftol, self._xtol = 1e-8 * N, 1e-11 * N, 1e-12
        else:
            tol, ftol, self._xtol = 1e-7 * N, 1e-7 * N, 1e-9
        if self.mu is not None:
            mu, e_lo = self.mu, self.e_lo
            if self._edge_ok(mu, e_lo):
                # with density when mu was kept last time (then this is likely the only pass);
                # over the trace rows when the last call had to re-solve mu
                dens, n, eb = self.pole_pass(mu, e_lo, want_density=not (self._trace and self._resolved))
                cnt = n - N
                if self.lag_mu and abs(cnt) < 0.25:
                    self.mu = mu
                    dens, eb = self._with_density(mu, e_lo, dens, eb)
                    return dens.reshape(cr.shape), eb, mu
                self._resolved = abs(cnt) > tol
                if abs(cnt) > tol:
                    mu, dens, eb = self._solve_mu(e_lo, N, ftol, start=(mu, cnt, dens, eb))
                self.mu = self._mu_last = mu
                dens, eb = self._with_density(mu, e_lo, dens, eb)
                return dens.reshape(cr.shape), eb, mu
        # cold path: new filter edge from the smallest window eigenvalue (inertia bisection,
        # bracketed around the previous one when there is one)
        if self._lam_min is not None:
            lam_min = self.min_eig(self._lam_min - 0.05, self._lam_min + 0.05, tol=1e-10)
        else:
            lam_min = self.min_eig(-1.0, 0.0, tol=1e-10)
        self._lam_min = lam_min
        e_lo = lam_min - self.margin
        lo = max(lam_min, e_lo + 1e-6)
        found = False
        if self._mu_last is not None and self._mu_last > lo:
            # the root of the (monotone) count is unique: start from the previous mu
            try:
                dens, n, eb = self.pole_pass(self._mu_last, e_lo, want_density=not self._trace)
                mu, dens, eb = self._solve_mu(e_lo, N, ftol, start=(self._mu_last, n - N, dens, eb))
                found = True
            except StaleMu:
                pass
        if not found:
            mu, dens, eb = self._solve_mu(e_lo, N, ftol, lo_start=lo)
        self.mu, self.e_lo = mu, e_lo
        self._mu_last = mu
        self._resolved = True
        dens, eb = self._with_density(mu, e_lo, dens, eb)
        return dens.reshape(cr.shape), eb, mu

    def _with_density(self, mu, e_lo, dens, eb):
        """The accepted pass's density, or (after trace-row passes) one density pass at mu."""
        if dens is not None:
            return dens, eb
        dens, _, eb = self.pole_pass(mu, e_lo)
        return dens, eb
