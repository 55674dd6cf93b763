"""The committed regression fixtures (tests/golden/oracle_l1.npz, written by
tests/golden/make_golden.py from the FP64 oracle): the oracle still produces them (1e-12
relative: the same code, possibly another platform's libm), and the library's host-side
cluster trees equal the fixture's permutations bit for bit."""
import os
import sys

import numpy as np
import pytest

import ngbem_gb300 as nb
from ngbem_gb300.meshes import icosphere

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import make_golden  # noqa: E402


@pytest.fixture(scope="module")
def golden():
    with np.load(os.path.join(GOLDEN, "oracle_l1.npz")) as z:
        return {k: z[k] for k in z.files}


def test_oracle_reproduces_the_fixtures(oracle, golden):
    now = make_golden.compute(oracle)
    assert set(now) == set(golden)
    for k, v in golden.items():
        if k.startswith("perm__"):
            assert np.array_equal(now[k], v), k
        else:
            assert now[k].shape == v.shape, k
            assert np.linalg.norm(now[k] - v) <= 1e-12 * np.linalg.norm(v), k


def test_host_trees_match_the_fixtures(golden):
    m = icosphere(1)
    for kind in ("P0", "P1", "RT0", "HCURL"):
        perm, _, _ = nb.cluster_tree(nb.TraceSpace(m, kind), 10)
        assert np.array_equal(perm, golden[f"perm__{kind}"]), kind
