"""Writes tests/golden/oracle_l1.npz: regression fixtures of the FP64 oracle on the level-1
icosphere (80 triangles), one entry per kernel / space / trace combination of the operator
path.  The reference itself cannot run here (it is an NGSolve add-on), so these vectors come
from the oracle: they pin it against accidental change, and they let the parity tests check
a fixed set of numbers.

For each combination: the dense Galerkin matrix (Sauter-Schwab order 4, regular order 3)
applied to three seeded vectors, shape (test ndof, 3).  Also the cluster-tree permutations of
the four spaces at leaf size 10.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from ngbem_gb300.meshes import icosphere  # noqa: E402
from oracle import pyoracle  # noqa: E402

CASES = [
    ("laplace_sl", "P0", "P0", "id", "id", 0.0),
    ("laplace_sl", "P1", "P1", "id", "id", 0.0),
    ("laplace_dl", "P1", "P0", "id", "id", 0.0),
    ("laplace_hs", "P1", "P1", "rot", "rot", 0.0),
    ("helmholtz_sl", "P0", "P0", "id", "id", 3.0),
    ("helmholtz_dl", "P1", "P1", "id", "id", 3.0),
    ("helmholtz_cf", "P1", "P1", "id", "id", 5.0),
    ("helmholtz_hs", "P1", "P1", "helm", "helm", 3.0),
    ("helmholtz_sl_dkappa", "P1", "P0", "id", "id", 3.0),
    ("maxwell_sl", "RT0", "RT0", "maxwell", "maxwell", 2.0),
    ("maxwell_sl", "HCURL", "HCURL", "maxwellcurl", "maxwellcurl", 2.0),
    ("maxwell_dl", "HCURL", "RT0", "rotatedtrace", "id", 2.0),
]
SEED = 20261203


def key(case):
    k, tr, te, e1, e2, _ = case
    return f"{k}__{tr}_{e1}__{te}_{e2}"


def inputs(n, cplx):
    r = np.random.default_rng(SEED)
    x = r.standard_normal((n, 3))
    return x + 1j * r.standard_normal((n, 3)) if cplx else x


def compute(oracle):
    m = icosphere(1)
    out = {}
    for case in CASES:
        k, tr, te, e1, e2, kap = case
        D = oracle.dense_matrix(k, m, tr, te, kappa=kap, trial_eval=e1, test_eval=e2, intorder_singular=4,
                                intorder_regular=3)
        out[key(case)] = D @ inputs(D.shape[1], np.iscomplexobj(D))
    for kind in ("P0", "P1", "RT0", "HCURL"):
        out[f"perm__{kind}"] = oracle.cluster_tree(m, kind, 10)[0]
    return out


if __name__ == "__main__":
    pyoracle.build()
    np.savez_compressed(os.path.join(HERE, "oracle_l1.npz"), **compute(pyoracle))
    print("wrote", os.path.join(HERE, "oracle_l1.npz"))
