"""Full-size workloads (the benchmark configurations) checked through
size-independent properties and an exact oracle sample:

* the dilation contains its input and the erosion lies inside it;
* repeated runs are bit-identical (deterministic kernels);
* a random sample of output columns equals the oracle's result for exactly
  those columns (vo_or_dilate_columns), bit for bit;
* brute force and separable agree on a sampled window.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import ogrid

pytestmark = pytest.mark.gpu


def _contains(big, small, cols):
    bo, bz = big
    so, sz = small
    for c in cols:
        b = bz[2 * bo[c]:2 * bo[c + 1]].reshape(-1, 2)
        for lo, hi in sz[2 * so[c]:2 * so[c + 1]].reshape(-1, 2):
            if lo > hi:
                continue
            assert np.any((b[:, 0] <= lo) & (hi <= b[:, 1])), f"column {c}: [{lo},{hi}] not covered"


@pytest.fixture(scope="module")
def spheres_cyl2048(vo):
    return vo.workload("spheres_cyl2048", seed=1)


@pytest.mark.parametrize("r", [32.0, 64.0])
def test_fullsize_dilation_sampled_exact(ctx, vo, oracle, spheres_cyl2048, r):
    grid, offs, z = spheres_cyl2048
    v = ctx.upload(grid, offs, z)
    out, t = ctx.morph(v, "dilation", r, "fast")
    got = ctx.download(out)
    out2, _ = ctx.morph(v, "dilation", r, "fast")
    again = ctx.download(out2)
    assert np.array_equal(got[0], again[0]) and np.array_equal(got[1], again[1])
    rng = np.random.default_rng(int(r))
    cols = np.unique(np.concatenate([rng.integers(0, grid.ncols, 400),
                                     [0, grid.nx - 1, grid.ncols - 1, grid.ncols - grid.nx]])).astype(np.int32)
    so, sz = oracle.dilate_columns(ogrid(oracle, grid), offs, z, r, cols)
    go, gz = got
    for i, c in enumerate(cols):
        a = gz[2 * go[c]:2 * go[c + 1]]
        b = sz[2 * so[i]:2 * so[i + 1]]
        assert np.array_equal(a, b), f"column {c}: GPU {a[:6]} vs oracle {b[:6]}"
    _contains(got, (offs, z), rng.integers(0, grid.ncols, 2000))


def test_fullsize_erosion_inside(ctx, vo, spheres_cyl2048):
    grid, offs, z = spheres_cyl2048
    v = ctx.upload(grid, offs, z)
    e, _ = ctx.morph(v, "erosion", 32.0, "fast")
    eo = ctx.download(e)
    rng = np.random.default_rng(3)
    _contains((offs, z), eo, rng.integers(0, grid.ncols, 3000))


def test_fullsize_plain_matches_fast(ctx, vo, spheres_cyl2048):
    """The FP64 separable kernels and the FP32-guarded kernel agree bit for bit
    on the full 2048^2 workload (radius 4 keeps the FP64 run short)."""
    grid, offs, z = spheres_cyl2048
    v = ctx.upload(grid, offs, z)
    a, _ = ctx.morph(v, "dilation", 4.0, "separable")
    b, _ = ctx.morph(v, "dilation", 4.0, "fast")
    ao, az = ctx.download(a)
    bo, bz = ctx.download(b)
    assert np.array_equal(ao, bo) and np.array_equal(az, bz)
