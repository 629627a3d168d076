"""lres_inertia_noalloc: window inertia counts for callers that cannot allocate device
memory (hosts that hand out all GPU memory from their own allocator, or loops that
cannot take cudaMalloc's device-wide synchronisation).  Called through the C ABI twice
in a row on caller-owned device arrays, its counts must equal those of lres_inertia and
the number of generalised eigenvalues of (H_W, S_W) below sigma from the oracle's
eigensolver (integers: exact).  Sizes beyond the fixed scratch, a window larger than the
nmax given and a NaN in one window are reported, not run through.  Collected last, so a
failure here comes after every other test."""
import numpy as np
import pytest

from golden_util import crystal, load

pytestmark = pytest.mark.gpu


def test_noalloc_inertia_matches_context_inertia():
    import torch
    from lresdft_gb300 import LResGPU, _lib, system
    g = load("cubic3")
    cr = crystal(g)
    b = system.LCAOBasis(cr)
    v = g["v"].reshape(cr.shape)
    s = LResGPU(b, cr.pos, R_w=float(g["R_w"]), M=int(g["M"]), precision="fp64")
    s.set_potential(v)
    # caller-side device arrays: dense column-major window blocks of H(v) and S
    H, S = b.H(v).tocsr(), b.S.tocsr()
    nW = np.array([len(W) for W in s.windows], np.int32)
    off = np.concatenate([[0], np.cumsum(nW.astype(np.int64) ** 2)]).astype(np.int64)
    Hd = np.empty(off[-1])
    Sd = np.empty(off[-1])
    for w, W in enumerate(s.windows):
        Hd[off[w]:off[w + 1]] = H[W][:, W].toarray().ravel(order="F")
        Sd[off[w]:off[w + 1]] = S[W][:, W].toarray().ravel(order="F")
    dev = torch.device("cuda", torch.cuda.current_device())
    t_n = torch.from_numpy(nW).to(dev)
    t_off = torch.from_numpy(off[:-1].copy()).to(dev)
    t_H = torch.from_numpy(Hd).to(dev)
    t_S = torch.from_numpy(Sd).to(dev)
    below = torch.full((len(nW),), -1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    lm = g["lam_min"]
    sigmas = [float(lm.min()) + 0.05, float(g["cold_mu"])]
    # the oracle's window spectra (scipy generalised eigh, as the reference's dsygvd)
    from scipy import linalg
    spectra = [linalg.eigh(Hd[off[w]:off[w + 1]].reshape(n, n, order="F"),
                           Sd[off[w]:off[w + 1]].reshape(n, n, order="F"), eigvals_only=True)
               for w, n in enumerate(nW)]
    for sigma in sigmas:                       # two calls in a row share the scratch array
        ref = s.inertia(sigma, per_window=True)
        orc = np.array([int(np.sum(lam < sigma)) for lam in spectra])
        gap = min(float(np.min(np.abs(lam - sigma))) for lam in spectra)
        assert gap > 1e-8                      # no eigenvalue at sigma: the counts are sharp
        _lib.check(_lib.lib.lres_inertia_noalloc(len(nW), t_n.data_ptr(), t_off.data_ptr(), t_H.data_ptr(),
                                                 t_S.data_ptr(), sigma, below.data_ptr(), int(nW.max()), stream))
        got = below.cpu().numpy()
        assert np.array_equal(got, ref), (sigma, got, ref)
        assert np.array_equal(got, orc), (sigma, got, orc)
    assert got.sum() > 0
    # sizes beyond the stated maximum are rejected, not run
    rc = _lib.lib.lres_inertia_noalloc(len(nW), t_n.data_ptr(), t_off.data_ptr(), t_H.data_ptr(), t_S.data_ptr(),
                                       0.0, below.data_ptr(), 513, stream)
    assert rc == -22 and b"exceed" in _lib.lib.lres_last_error()
    # a window larger than the nmax given: found by the kernel, reported as LRES_EINVAL
    rc = _lib.lib.lres_inertia_noalloc(len(nW), t_n.data_ptr(), t_off.data_ptr(), t_H.data_ptr(), t_S.data_ptr(),
                                       sigmas[0], below.data_ptr(), int(nW.max()) - 1, stream)
    assert rc == -22 and b"larger than nmax" in _lib.lib.lres_last_error()
    # a NaN in one window's H: LRES_ENUMERIC, not a count
    t_Hbad = t_H.clone()
    t_Hbad[int(off[3]) + 1] = float("nan")
    rc = _lib.lib.lres_inertia_noalloc(len(nW), t_n.data_ptr(), t_off.data_ptr(), t_Hbad.data_ptr(),
                                       t_S.data_ptr(), sigmas[0], below.data_ptr(), int(nW.max()), stream)
    assert rc == -33 and b"pivot" in _lib.lib.lres_last_error()
    # and the next clean call is unaffected by the earlier ones
    _lib.check(_lib.lib.lres_inertia_noalloc(len(nW), t_n.data_ptr(), t_off.data_ptr(), t_H.data_ptr(),
                                             t_S.data_ptr(), sigmas[1], below.data_ptr(), int(nW.max()), stream))
    assert np.array_equal(below.cpu().numpy(), s.inertia(sigmas[1], per_window=True))
    s.close()
