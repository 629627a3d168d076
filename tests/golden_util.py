"""Helpers shared by tests: load golden fixtures and rebuild their systems."""
import os

import numpy as np

from lresdft_gb300 import system

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def crystal(g):
    pos = g["pos"]
    return system.Crystal(pos.copy(), np.ones(len(pos)), g["cell"].copy(), tuple(int(s) for s in g["shape"]),
                          float(g["rc"]))


def check_basis(b, g, prefix="b_"):
    X = b.Xr
    assert b.nb == int(g[prefix + "nb"])
    assert X.nnz == int(g[prefix + "X_nnz"])
    assert abs(X.data.sum() - g[prefix + "X_sum"]) < 1e-9
    assert abs((X.data ** 2).sum() - g[prefix + "X_sumsq"]) < 1e-8
    S, T = b.S.tocsr(), b.T.tocsr()
    assert S.nnz == int(g[prefix + "S_nnz"])
    Sd = np.asarray(S[g[prefix + "S_row"], g[prefix + "S_col"]]).ravel()
    Td = np.asarray(T[g[prefix + "T_row"], g[prefix + "T_col"]]).ravel()
    assert np.max(np.abs(Sd - g[prefix + "S_val"])) < 1e-14
    assert np.max(np.abs(Td - g[prefix + "T_val"])) < 1e-12
    assert np.array_equal(np.asarray(b.atom_of_fn), g[prefix + "atom_of_fn"])
