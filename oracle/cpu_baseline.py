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
