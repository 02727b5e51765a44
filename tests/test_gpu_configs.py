"""Every benchmark configuration at the size it is run, checked against the
oracle bit for bit (endpoint tolerance 0, so well inside the 1e-9 dexel of the
plain method and the 1e-5 of the FP32 variant):

* 1024^2, 4096 spheres, all four ops at r = 32: whole volumes;
* 2048^2 spheres + cylinders: erosion, opening and closing at r = 32 on
  sampled columns (the dilations at r = 32 and 64 are in test_gpu_fullsize);
* the 256-volume batch of the benchmark (sides 64-1024, r in [2, 64], mixed
  ops) through one batch plan: every volume, whole for sides up to 128 and on
  sampled columns above;
* 4096^2, 20000 cylinders, dilation at r = 16 (the learned-sizing
  configuration): the single-volume method and the learned batch plan on
  sampled columns.

Sampled columns always include the grid's corners and edge midpoints, where
the erosion's border and the clipped lattice discs act.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import assert_same, ogrid

pytestmark = pytest.mark.gpu

OPS = ["dilation", "erosion", "opening", "closing"]


def sample_columns(g, n, seed):
    rng = np.random.default_rng(seed)
    nx, ny = g.nx, g.ny
    edges = [0, nx - 1, nx * (ny - 1), nx * ny - 1, nx // 2, nx * (ny // 2), nx * (ny // 2) + nx - 1,
             nx * (ny - 1) + nx // 2]
    return np.unique(np.concatenate([rng.integers(0, nx * ny, n), edges])).astype(np.int32)


def check_columns(got, want_cols, cols, what):
    go, gz = got
    so, sz = want_cols
    for i, c in enumerate(cols):
        a = gz[2 * go[c]:2 * go[c + 1]]
        b = sz[2 * so[i]:2 * so[i + 1]]
        assert np.array_equal(a, b), f"{what}: column {c}: GPU {a[:6]} vs oracle {b[:6]}"


def learned_sizer(ctx):
    from voroffset_gb300.train_sizer import WEIGHTS, load
    return load(ctx) if os.path.exists(WEIGHTS) else None


@pytest.mark.parametrize("op", OPS)
def test_config_spheres1024_all_ops_whole_volume(ctx, vo, oracle, op):
    grid, offs, z = vo.workload("spheres1024", seed=1)
    want = oracle.morph(ogrid(oracle, grid), offs, z, 32.0, op)
    v = ctx.upload(grid, offs, z)
    single, _ = ctx.morph(v, op, 32.0, "fast")
    outs, _ = ctx.morph_batched([v], [op], [32.0], "fast")
    for name, out in (("fast", single), ("batched", outs[0])):
        assert_same(ctx.download(out), want, tol=0.0, what=f"spheres1024 {op} r=32 {name}")
        out.free()
    v.free()


@pytest.fixture(scope="module")
def spheres_cyl2048(vo):
    return vo.workload("spheres_cyl2048", seed=1)


@pytest.mark.parametrize("op", ["erosion", "opening", "closing"])
def test_config_spheres_cyl2048_ops_sampled(ctx, vo, oracle, spheres_cyl2048, op):
    grid, offs, z = spheres_cyl2048
    cols = sample_columns(grid, 120 if op == "erosion" else 40, seed=OPS.index(op))
    want = oracle.morph_columns(ogrid(oracle, grid), offs, z, 32.0, op, cols)
    v = ctx.upload(grid, offs, z)
    single, _ = ctx.morph(v, op, 32.0, "fast")
    check_columns(ctx.download(single), want, cols, f"spheres_cyl2048 {op} r=32 fast")
    single.free()
    plan = ctx.batch([v], [op], [32.0], "fast")
    plan.run()
    out = plan.outputs()[0]
    check_columns(ctx.download(out), want, cols, f"spheres_cyl2048 {op} r=32 batch plan")
    out.free()
    plan.free()
    v.free()


def test_config_batch256_every_volume(ctx, vo, oracle):
    import bench
    items = bench.batch_volumes(vo, 256, seed=7)
    sizer = learned_sizer(ctx)
    ctx.set_sizer(sizer)
    vols = [ctx.upload(g, o, z) for g, o, z, _, _ in items]
    plan = ctx.batch(vols, [it[4] for it in items], [it[3] for it in items], "fast")
    plan.run()
    outs = plan.outputs()
    ctx.set_sizer(None)
    if sizer is not None:
        sizer.free()
    checked_whole = checked_sampled = 0
    for i, ((g, o, z, r, op), out) in enumerate(zip(items, outs)):
        got = ctx.download(out)
        out.free()
        og = ogrid(oracle, g)
        what = f"volume {i}: {g.nx}^2 {op} r={r}"
        if g.nx <= 128:
            assert_same(got, oracle.morph(og, o, z, r, op), tol=0.0, what=what)
            checked_whole += 1
        else:
            # the first op of an opening / closing is evaluated on each sample's lattice neighbourhood
            n = 10 if op in ("dilation", "erosion") else (3 if r <= 32 else 1)
            cols = sample_columns(g, n, seed=i)
            check_columns(got, oracle.morph_columns(og, o, z, r, op, cols), cols, what)
            checked_sampled += 1
    plan.free()
    for v in vols:
        v.free()
    assert checked_whole + checked_sampled == 256 and checked_whole > 50


def test_config_cyl4096_r16_sampled(ctx, vo, oracle):
    grid, offs, z = vo.workload("cyl4096", seed=1)
    cols = sample_columns(grid, 300, seed=16)
    want = oracle.dilate_columns(ogrid(oracle, grid), offs, z, 16.0, cols)
    v = ctx.upload(grid, offs, z)
    del offs, z
    single, _ = ctx.morph(v, "dilation", 16.0, "fast")
    check_columns(ctx.download(single), want, cols, "cyl4096 r=16 fast")
    single.free()
    sizer = learned_sizer(ctx)
    ctx.set_sizer(sizer)
    plan = ctx.batch([v], ["dilation"], [16.0], "fast")
    plan.run()
    st = plan.stats()
    out = plan.outputs()[0]
    check_columns(ctx.download(out), want, cols, "cyl4096 r=16 learned batch plan")
    out.free()
    plan.free()
    ctx.set_sizer(None)
    if sizer is not None:
        sizer.free()
        assert st["learned"] == 1
    v.free()
