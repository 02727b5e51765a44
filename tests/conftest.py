"""Shared fixtures. GPU tests carry @pytest.mark.gpu and run only with -m gpu."""
from __future__ import annotations

import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "*.npz")))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build(ref=None)
    return O


@pytest.fixture(scope="session")
def vo():
    import voroffset_gb300 as V
    V.lib(build_if_missing=True)
    return V


@pytest.fixture(scope="session")
def ctx(vo):
    c = vo.Context(0)
    yield c
    c.close()


def load_golden(path):
    d = np.load(path)
    import voroffset_gb300 as V
    grid = V.Grid(int(d["nx"]), int(d["ny"]), tuple(d["origin"]), tuple(d["extent"]), float(d["spacing"]),
                  int(d["padding"]))
    return grid, d


def ogrid(O, g):
    return O.Grid(g.nx, g.ny, g.origin, g.extent, g.spacing, g.padding)


def assert_same(a, b, tol=0.0, what=""):
    """Exact per-column segment counts; endpoints equal within tol."""
    oa, za = a
    ob, zb = b
    oa, ob = np.asarray(oa), np.asarray(ob)
    assert oa.shape == ob.shape, f"{what}: grid sizes differ"
    ca, cb = np.diff(oa), np.diff(ob)
    bad = np.nonzero(ca != cb)[0]
    assert bad.size == 0, f"{what}: {bad.size} columns with different segment counts, first {bad[:8]}"
    za, zb = np.asarray(za), np.asarray(zb)
    assert za.shape == zb.shape
    if za.size:
        err = float(np.max(np.abs(za - zb)))
        assert err <= tol, f"{what}: max endpoint error {err} > {tol}"
