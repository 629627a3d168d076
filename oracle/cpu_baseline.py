"""TEST / BASELINE INFRASTRUCTURE ONLY — times the reference's CPU algorithm for the
window pass on the host cores.  Used by bench.py's CPU-baseline and reference legs,
never by the product.

The timed work is one window pass of the reference's production route,
``_lrft_cpp.lrft_windows`` (src/lrft_cpp.cpp:148-196): for every window, gather
dense H_W and S_W, the generalised eigenpairs below c + 1.5 R with LAPACK dsygvx
(scipy's bundled OpenBLAS here), Y = X[own, W] U, occupation r_M and the owned-point
density.  Windows are spread over worker processes (spawn start method, one
single-threaded BLAS per process), like the reference's OpenMP loop over windows
with one OpenBLAS thread each.  The result is expressed in the GPU metric's unit:
(windows x M/2) / wall time, i.e. window-pole solves per second that the eigen route
replaces.  The reference's own pole route (benchmarks/window_resolvent_vs_eig.py:58-65,
one scipy.linalg.solve per window and pole) is timed on a small sample as well.

``scf_window`` times the reference's SCF (lrft/lcao3d.py:237-284 with the LRFTLCAOCpp
solver protocol, lrft/lcao3d.py:340-456, restated by oracle.lrft_oracle) over a fixed number
of iterations, wrapping the solver like the reference's ``Timed`` helper
(benchmarks/scf3d_large.py:35-45): H(v) by scipy in the main process (single-threaded, as in
the reference), every window pass spread over worker processes.
"""
from __future__ import annotations

import multiprocessing as mp
import os
import tempfile
import time

import numpy as np

_W = {}


def _init(path):
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    from scipy import sparse
    ld = lambda n: np.load(os.path.join(path, n + ".npy"), mmap_mode="r")  # noqa: E731
    nb, ng = int(ld("dims")[0]), int(ld("dims")[1])
    _W["H"] = sparse.csr_matrix((ld("Hv"), ld("Hi"), ld("Hp")), shape=(nb, nb))
    _W["S"] = sparse.csr_matrix((ld("Sv"), ld("Si"), ld("Sp")), shape=(nb, nb))
    _W["X"] = sparse.csr_matrix((ld("Xv"), ld("Xi"), ld("Xp")), shape=(ng, nb))
    for k in ("Wflat", "Woff", "Oflat", "Ooff", "par"):
        _W[k] = np.asarray(ld(k))


def _windows(ws):
    from scipy import linalg
    H, S, X = _W["H"], _W["S"], _W["X"]
    Wf, Wo, Of, Oo = _W["Wflat"], _W["Woff"], _W["Oflat"], _W["Ooff"]
    mu, e_lo, M, dV = _W["par"]
    M = int(M)
    c, R = 0.5 * (mu + e_lo), 0.5 * (mu - e_lo)
    upper = c + 1.5 * R
    out = 0.0
    for w in ws:
        W = Wf[Wo[w]:Wo[w + 1]]
        own = Of[Oo[w]:Oo[w + 1]]
        HW, SW = H[W][:, W].toarray(), S[W][:, W].toarray()
        lam, U = linalg.eigh(HW, SW, subset_by_value=(-np.inf, upper), driver="gvx")
        Y = X[own][:, W] @ U
        u = (lam - c) / R
        with np.errstate(over="ignore"):
            occ = 1.0 / (1.0 + u ** M)
        out += float(((Y * Y) @ occ).sum() * dV)
    return out


def _pole_windows(ws):
    from scipy import linalg
    H, S, X = _W["H"], _W["S"], _W["X"]
    Wf, Wo, Of, Oo = _W["Wflat"], _W["Woff"], _W["Oflat"], _W["Ooff"]
    mu, e_lo, M, dV = _W["par"]
    M = int(M)
    c, R = 0.5 * (mu + e_lo), 0.5 * (mu - e_lo)
    zeta = np.exp(1j * np.pi * (2 * np.arange(M // 2) + 1) / M)
    out = 0.0
    for w in ws:
        W = Wf[Wo[w]:Wo[w + 1]]
        own = Of[Oo[w]:Oo[w + 1]]
        HW, SW = H[W][:, W].toarray(), S[W][:, W].toarray()
        F = X[own][:, W].toarray().T
        for z, wt in zip(c + R * zeta, R * zeta / M):
            Y = linalg.solve(z * SW - HW, F.astype(complex))
            out += float(np.real(wt * np.sum(F * Y)))
    return out


def run(H, S, X, Wflat, Woff, Oflat, Ooff, mu, e_lo, M, dV, workers=None, pole_sample=16):
    """Times one eigen-route window pass over all windows on `workers` processes and the
    scipy pole route on `pole_sample` windows; returns a dict of rates."""
    from scipy import sparse
    workers = workers or len(os.sched_getaffinity(0))
    H, S, X = sparse.csr_matrix(H), sparse.csr_matrix(S), sparse.csr_matrix(X)
    nwin = len(Woff) - 1
    with tempfile.TemporaryDirectory(prefix="lres_cpu_") as d:
        arrs = dict(dims=np.array([H.shape[0], X.shape[0]]), Hp=H.indptr, Hi=H.indices, Hv=H.data, Sp=S.indptr,
                    Si=S.indices, Sv=S.data, Xp=X.indptr, Xi=X.indices, Xv=X.data, Wflat=Wflat, Woff=Woff,
                    Oflat=Oflat, Ooff=Ooff, par=np.array([mu, e_lo, M, dV], float))
        for k, a in arrs.items():
            np.save(os.path.join(d, k + ".npy"), np.ascontiguousarray(a))
        env_before = os.environ.get("OPENBLAS_NUM_THREADS")
        os.environ["OPENBLAS_NUM_THREADS"] = "1"
        ctx = mp.get_context("spawn")
        try:
            with ctx.Pool(workers, initializer=_init, initargs=(d,)) as pool:
                # largest windows first, round-robin chunks
                order = np.argsort(-(np.diff(Woff)), kind="stable")
                chunks = [order[i::workers * 4].tolist() for i in range(workers * 4)]
                pool.map(_windows, [[int(order[0])]] * workers)          # warm-up (imports, page-in)
                t = time.perf_counter()
                pool.map(_windows, chunks)
                t_eig = time.perf_counter() - t
                samp = order[:: max(1, nwin // pole_sample)][:pole_sample].tolist()
                pchunks = [samp[i::workers] for i in range(workers) if samp[i::workers]]
                t = time.perf_counter()
                pool.map(_pole_windows, pchunks)
                t_pole = time.perf_counter() - t
        finally:
            if env_before is None:
                os.environ.pop("OPENBLAS_NUM_THREADS", None)
            else:
                os.environ["OPENBLAS_NUM_THREADS"] = env_before
    P = M // 2
    return dict(
        eig_rate=nwin * P / t_eig, eig_wall=t_eig, nwin=nwin, workers=workers,
        pole_rate=len(samp) * P / t_pole, pole_wall=t_pole, pole_windows=len(samp),
    )


# ---------------------------------------------------------------------------
# SCF seconds per iteration of the reference algorithm on the host cores
# ---------------------------------------------------------------------------

_S = {}


def _init_scf(path):
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    from scipy import sparse
    ld = lambda n: np.load(os.path.join(path, n + ".npy"), mmap_mode="r")  # noqa: E731
    nb, ng = int(ld("dims")[0]), int(ld("dims")[1])
    _S["path"], _S["nb"] = path, nb
    _S["S"] = sparse.csr_matrix((ld("Sv"), ld("Si"), ld("Sp")), shape=(nb, nb))
    _S["X"] = sparse.csr_matrix((ld("Xv"), ld("Xi"), ld("Xp")), shape=(ng, nb))
    for k in ("Wflat", "Woff", "Oflat", "Ooff", "dV"):
        _S[k] = np.asarray(ld(k))


def _scf_windows(args):
    """Eigen route over some windows (src/lrft_cpp.cpp:148-196): owned densities (no spin
    factor), eigenvalues and owned weights."""
    from scipy import linalg, sparse
    ws, tag, mu, e_lo, M, upper, want = args
    if _S.get("Htag") != tag:
        ld = lambda n: np.load(os.path.join(_S["path"], f"{n}_{tag}.npy"), mmap_mode="r")  # noqa: E731
        nb = _S["nb"]
        _S["H"] = sparse.csr_matrix((np.asarray(ld("Hv")), np.asarray(ld("Hi")), np.asarray(ld("Hp"))),
                                    shape=(nb, nb))
        _S["Htag"] = tag
    H, S, X = _S["H"], _S["S"], _S["X"]
    Wf, Wo, Of, Oo, dV = _S["Wflat"], _S["Woff"], _S["Oflat"], _S["Ooff"], float(_S["dV"][0])
    c0, R = 0.5 * (mu + e_lo), 0.5 * (mu - e_lo)
    out = []
    for w in ws:
        W = Wf[Wo[w]:Wo[w + 1]]
        own = Of[Oo[w]:Oo[w + 1]]
        HW, SW = H[W][:, W].toarray(), S[W][:, W].toarray()
        if np.isfinite(upper):
            lam, U = linalg.eigh(HW, SW, subset_by_value=(-np.inf, upper), driver="gvx")
        else:
            lam, U = linalg.eigh(HW, SW, driver="gvd")
        Y = X[own][:, W] @ U
        c = np.sum(Y * Y, axis=0) * dV
        d = None
        if want:
            with np.errstate(over="ignore"):
                occ = 1.0 / (1.0 + ((lam - c0) / R) ** M)
            d = (Y * Y) @ occ
        out.append((w, d, lam, c))
    return out


class EigenPool:
    """``window_pass`` of the eigen route over worker processes (spawn start method, one
    single-threaded BLAS each), for oracle.lrft_oracle.LResEigenOracle(pool=...)."""

    def __init__(self, basis, windows, own, workers=None):
        from scipy import sparse
        self.workers = workers or len(os.sched_getaffinity(0))
        self.ng = basis.cr.ng
        self.dir = tempfile.TemporaryDirectory(prefix="lres_scf_")
        S, X = sparse.csr_matrix(basis.S), sparse.csr_matrix(basis.Xr)
        Woff = np.concatenate([[0], np.cumsum([len(W) for W in windows])]).astype(np.int64)
        Ooff = np.concatenate([[0], np.cumsum([len(o) for o in own])]).astype(np.int64)
        self.Oflat = np.concatenate(own).astype(np.int64)
        self.Ooff = Ooff
        arrs = dict(dims=np.array([S.shape[0], X.shape[0]]), Sp=S.indptr, Si=S.indices, Sv=S.data, Xp=X.indptr,
                    Xi=X.indices, Xv=X.data, Wflat=np.concatenate(windows).astype(np.int64), Woff=Woff,
                    Oflat=self.Oflat, Ooff=Ooff, dV=np.array([basis.cr.dV]))
        for k, a in arrs.items():
            np.save(os.path.join(self.dir.name, k + ".npy"), np.ascontiguousarray(a))
        order = np.argsort(-np.diff(Woff), kind="stable")
        self.chunks = [order[i::self.workers * 4].tolist() for i in range(self.workers * 4)]
        self.nwin = len(windows)
        self.calls = 0
        self.pool = mp.get_context("spawn").Pool(self.workers, initializer=_init_scf, initargs=(self.dir.name,))

    def window_pass(self, H, mu, e_lo, M, upper, want_density):
        from scipy import sparse
        H = sparse.csr_matrix(H)
        self.calls += 1
        tag = self.calls
        for k, a in (("Hp", H.indptr), ("Hi", H.indices), ("Hv", H.data)):
            np.save(os.path.join(self.dir.name, f"{k}_{tag}.npy"), np.ascontiguousarray(a))
        res = self.pool.map(_scf_windows, [(ch, tag, mu, e_lo, M, upper, want_density) for ch in self.chunks])
        per = {w: (d, lam, c) for part in res for (w, d, lam, c) in part}
        dens = np.zeros(self.ng) if want_density else None
        lams, cs = [], []
        for w in range(self.nwin):
            d, lam, c = per[w]
            if want_density:
                dens[self.Oflat[self.Ooff[w]:self.Ooff[w + 1]]] = d
            lams.append(lam)
            cs.append(c)
        for k in ("Hp", "Hi", "Hv"):
            os.unlink(os.path.join(self.dir.name, f"{k}_{tag}.npy"))
        return dens, np.concatenate(lams), np.concatenate(cs)

    def close(self):
        self.pool.close()
        self.pool.join()
        self.dir.cleanup()


class Timed:
    """Records the wall time of every density call of a solver (the reference's
    benchmarks/scf3d_large.py:35-45 wrapper)."""

    def __init__(self, solver):
        self.s, self.times = solver, []

    def density(self, v):
        t = time.perf_counter()
        out = self.s.density(v)
        self.times.append(time.perf_counter() - t)
        return out


def scf_window(cr, basis, vion, R_w, M, iters, workers=None):
    """The reference's SCF (Pulay mixer, mix 0.4, ndiis 6) over a fixed window of `iters`
    iterations from the uniform start, eigen-route solver with its window passes on
    `workers` processes.  Returns s/iter (median of iterations 3..end, the whole iteration:
    LDA + Hartree + H(v) + density call + mixing), the density-call times, passes, energy."""
    from . import lrft_oracle as orc
    pool = None
    try:
        t = time.perf_counter()
        solver = orc.LResEigenOracle(basis, cr.pos, R_w=R_w, M=M)
        pool = EigenPool(basis, solver.windows, solver.own, workers)
        solver.pool = pool
        setup = time.perf_counter() - t
        timed = Timed(solver)
        # whole iterations: each density call starts at a mark, the driver's own work (LDA,
        # Hartree, mixing) sits between consecutive marks
        marks = []
        inner = timed.density

        class _Marked:
            def density(self, v):
                marks.append(time.perf_counter())
                return inner(v)
        t0 = time.perf_counter()
        r = orc.scf_lcao(cr, _Marked(), tol=1e-12, maxiter=iters, vion=vion)
        t_end = time.perf_counter()
        marks.append(t_end)
        it_times = [marks[i + 1] - marks[i] for i in range(len(marks) - 1)]
        sel = it_times[2:] if len(it_times) > 2 else it_times
        return dict(s_per_iter=float(np.median(sel)), iteration_s=[round(x, 3) for x in it_times],
                    density_call_s=[round(x, 3) for x in timed.times], passes=solver.passes,
                    energy=float(r["energy"]), workers=pool.workers, setup_s=round(setup, 2),
                    wall_s=round(t_end - t0, 2))
    finally:
        if pool is not None:
            pool.close()
