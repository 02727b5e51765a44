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


@pytest.mark.parametrize("op", ["dilation", "erosion", "opening", "closing"])
def test_config_spheres1024_all_ops_fast_equals_plain(ctx, vo, op):
    """1024^2 grid, 4096 spheres (radii 4-40), r = 32: the FP32-guarded method,
    single-volume and as a batch plan, equals the FP64 plain method bit for bit
    for every operation (the plain method equals the oracle on the parity
    suites)."""
    grid, offs, z = vo.workload("spheres1024", seed=1)
    v = ctx.upload(grid, offs, z)
    a, _ = ctx.morph(v, op, 32.0, "separable")
    b, _ = ctx.morph(v, op, 32.0, "fast")
    outs, t = ctx.morph_batched([v], [op], [32.0], "fast")
    ao, az = ctx.download(a)
    for other in (b, outs[0]):
        oo, oz = ctx.download(other)
        assert np.array_equal(ao, oo) and np.array_equal(az, oz), op


def test_config_torus_dexelize_and_dilate(ctx, vo, oracle):
    """The torus configuration: 256 x 64 quads (32768 triangles) displaced by
    seeded noise, -n 256 -p 10, dilation r = 8: the GPU rasteriser equals the
    oracle's, and so do the dilations (FP64 and FP32 methods), bit for bit."""
    verts, tris = vo.synth_torus(256, 64, 0.30, 0.10, 0.01, seed=1)
    og, offs, z = oracle.dexelize(verts, tris, num_dexels=256, padding=10)
    v = ctx.dexelize(verts, tris, num_dexels=256, padding=10)
    got = ctx.download(v)
    assert np.array_equal(got[0], offs) and np.array_equal(got[1], z)
    want = oracle.morph(og, offs, z, 8.0, "dilation")
    for method in ("separable", "fast"):
        out, _ = ctx.morph(v, "dilation", 8.0, method)
        o, zz = ctx.download(out)
        assert np.array_equal(o, want[0]) and np.array_equal(zz, want[1]), method
    assert ctx.xor_volume(out, out) == 0.0
