"""GB300 (sm_103a) LRes-DFT LCAO window solve: a drop-in for the reference's
``LRFTLCAOCpp`` solver (albert-hzbn/LResDFT, lrft/lcao3d.py) on one GPU.

``system`` (host geometry/basis set-up) imports without the CUDA library; the solver
and SCF modules load liblres_gb300.so and fail loudly if it was not built.
"""
__version__ = "0.1.0"


def __getattr__(name):
    if name in ("LResGPU", "StaleMu", "window_setup"):
        from . import solver
        return getattr(solver, name)
    if name == "scf_lcao":
        from . import scf
        return scf.scf_lcao
    raise AttributeError(name)
