"""Generate the golden vectors under tests/golden/ by running the REFERENCE's own code
(albert-hzbn/LResDFT: lrft.three_d, lrft.lcao3d and the C++ back end src/lrft_cpp.cpp
compiled by oracle/build_ref.sh).  Needs the reference's source tree, named by the
LRES_REFERENCE_ROOT environment variable:

    export LRES_REFERENCE_ROOT=<reference tree>
    sh oracle/build_ref.sh && python tests/golden/make_golden.py

Geometries are produced by lresdft_gb300.system (identical conventions to the
reference generators) and handed to the reference's Crystal / LCAOBasis, so the
fixtures also pin that module.  Outputs (npz, a few hundred KB in total):

  cubic3.npz   3x3x3 simple-cubic H2, a=4.5, bond 1.4 along z, default basis,
               one window per atom, R_w=8, M=64 (54 electrons)
  jit2.npz     2x2x2 h2_crystal (normal jitter 0.15, seed 0), same settings (16 e)
  jit8.npz     8x8x8 H2, uniform jitter 0.1, random axes, seed 0, same settings
               (1024 electrons): one cold density call, sampled
"""
from __future__ import annotations

import hashlib
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import refimport  # noqa: E402
from lresdft_gb300 import system  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
NTHREADS = int(os.environ.get("GOLDEN_THREADS", os.cpu_count() or 1))


def ref_crystal(td, cr):
    return td.Crystal(cr.pos.copy(), cr.Z.copy(), cr.cell.copy(), tuple(cr.shape), cr.rc)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()[:16]


def basis_record(b, prefix="b_"):
    X = b.Xr
    S, T = b.S.tocsr(), b.T.tocsr()
    rng = np.random.default_rng(123)
    k = rng.integers(0, S.nnz, 2000)
    Sc = S.tocoo()
    Tc = T.tocoo()
    return {
        prefix + "nb": b.nb, prefix + "X_nnz": X.nnz,
        prefix + "X_sum": X.data.sum(), prefix + "X_sumsq": (X.data ** 2).sum(),
        prefix + "X_indptr_sha": sha(X.indptr.astype(np.int64)),
        prefix + "S_nnz": S.nnz, prefix + "S_sum": S.data.sum(), prefix + "T_sum": T.data.sum(),
        prefix + "S_row": Sc.row[k], prefix + "S_col": Sc.col[k], prefix + "S_val": Sc.data[k],
        prefix + "T_row": Tc.row[k], prefix + "T_col": Tc.col[k], prefix + "T_val": Tc.data[k],
        prefix + "atom_of_fn": np.asarray(b.atom_of_fn, np.int32),
    }


def owner_of(L, ng):
    owner = np.empty(ng, np.int32)
    for B, o in enumerate(L.own):
        owner[o] = B
    return owner


def small_case(name, cr, M=64, R_w=8.0, scf=True):
    td, lc = refimport.load()
    rcr = ref_crystal(td, cr)
    t = time.time()
    b = lc.LCAOBasis(rcr)
    d0 = np.full(rcr.shape, rcr.n_elec / (rcr.ng * rcr.dV))
    vion = td.ion_potential(rcr)
    v = vion + td.hartree(rcr, d0) + td.lda_xc(d0)[1]
    rec = dict(pos=cr.pos, cell=cr.cell, shape=np.array(cr.shape), rc=cr.rc, M=M, R_w=R_w,
               vion=vion.ravel(), v=v.ravel())
    rec.update(basis_record(b))
    C = lc.LRFTLCAOCpp(b, rcr.pos.copy(), R_w=R_w, M=M, nthreads=NTHREADS, reuse_vectors=False)
    rec["owner"] = owner_of(C, rcr.ng)
    rec["nW"] = np.array(C.nW, np.int32)
    rec["Wflat"] = C.Wflat.astype(np.int32)
    rec["Woff"] = C.Woff
    # cold call, then a warm call at a perturbed potential with mu forced off (mu re-solve)
    n1, e1, mu1 = C.density(v)
    rec.update(cold_dens=n1.ravel(), cold_eband=e1, cold_mu=mu1, cold_elo=C.e_lo, cold_passes=C.passes)
    C.mu += 0.02
    n2, e2, mu2 = C.density(0.999 * v)
    rec.update(warm_dens=n2.ravel(), warm_eband=e2, warm_mu=mu2, warm_elo=C.e_lo)
    # a warm call that keeps mu (count within tolerance): same potential again
    p0 = C.passes
    n3, e3, mu3 = C.density(0.999 * v)
    rec.update(keep_dens=n3.ravel(), keep_eband=e3, keep_mu=mu3, keep_passes=C.passes - p0)
    # the pure-Python reference solver on the first potential
    npy, epy, mupy = lc.LRFTLCAO(b, rcr.pos.copy(), R_w=R_w, M=M).density(v)
    rec.update(py_dens=npy.ravel(), py_eband=epy, py_mu=mupy)
    # window minimum eigenvalues of the first potential (for inertia checks)
    from scipy import linalg
    H, S = b.H(v), b.S
    rec["lam_min"] = np.array([linalg.eigh(H[W][:, W].toarray(), S[W][:, W].toarray(),
                                           eigvals_only=True, subset_by_index=(0, 0))[0] for W in C.windows])
    if scf:
        for reuse in (False, True):
            s = lc.LRFTLCAOCpp(b, rcr.pos.copy(), R_w=R_w, M=M, nthreads=NTHREADS, reuse_vectors=reuse)
            r = lc.scf_lcao(rcr, s, tol=1e-8, maxiter=60)
            tag = "scf_reuse" if reuse else "scf"
            rec.update({tag + "_energy": r["energy"], tag + "_iterations": r["iterations"],
                        tag + "_converged": r["converged"], tag + "_mu": s.mu, tag + "_eband": r["eband"]})
            if not reuse:
                rec["scf_dens_in"] = r["dens_in"].ravel()
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **rec)
    print(name, "done", f"{time.time() - t:.1f}s", {k: rec[k] for k in rec if k.startswith(("cold_e", "cold_mu", "scf_e", "scf_it"))})


def large_case(name="jit8"):
    td, lc = refimport.load()
    cr = system.jittered_h2((8, 8, 8), a=4.5, bond=1.4, pts_per_cell=8, jitter=0.1, seed=0)
    rcr = ref_crystal(td, cr)
    t = time.time()
    b = lc.LCAOBasis(rcr)
    print("basis", time.time() - t, flush=True)
    d0 = np.full(rcr.shape, rcr.n_elec / (rcr.ng * rcr.dV))
    vion = td.ion_potential(rcr)
    v = vion + td.hartree(rcr, d0) + td.lda_xc(d0)[1]
    print("v", time.time() - t, flush=True)
    C = lc.LRFTLCAOCpp(b, rcr.pos.copy(), R_w=8.0, M=64, nthreads=NTHREADS, reuse_vectors=False)
    print("setup", time.time() - t, flush=True)
    n1, e1, mu1 = C.density(v)
    print("density", time.time() - t, flush=True)
    rng = np.random.default_rng(5)
    samp = np.sort(rng.choice(rcr.ng, 8192, replace=False))
    rec = dict(pos=cr.pos, cell=cr.cell, shape=np.array(cr.shape), rc=cr.rc, M=64, R_w=8.0,
               v_sum=v.sum(), v_sumsq=(v ** 2).sum(), v_sample=v.ravel()[samp], vion_sum=vion.sum(),
               sample=samp, dens_sample=n1.ravel()[samp], dens_sum=n1.sum(), dens_sumsq=(n1 ** 2).sum(),
               eband=e1, mu=mu1, e_lo=C.e_lo, nW=np.array(C.nW, np.int32),
               nown=np.array([len(o) for o in C.own], np.int32), owner_sha=sha(owner_of(C, rcr.ng)))
    rec.update(basis_record(b))
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **rec)
    print(name, "done", f"{time.time() - t:.1f}s", e1, mu1, C.e_lo)


if __name__ == "__main__":
    which = sys.argv[1:] or ["cubic3", "jit2", "jit8"]
    if "jit2" in which:
        small_case("jit2", system.h2_crystal((2, 2, 2)))
    if "cubic3" in which:
        small_case("cubic3", system.cubic_h2((3, 3, 3)))
    if "jit8" in which:
        large_case()
