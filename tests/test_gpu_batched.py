"""Batched execution (vo_morph_batched with the fast method): volumes of uneven
grids, radii and operations in shared persistent launches. Every output must
equal the oracle's result for that volume alone, bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import assert_same, ogrid

pytestmark = pytest.mark.gpu

OPS = ["dilation", "erosion", "opening", "closing"]


def _batch(vo, n, seed):
    rng = np.random.default_rng(seed)
    items = []
    for i in range(n):
        side = int(rng.choice([24, 40, 64, 96]))
        spec = vo.SynthSpec(side, n_spheres=int(rng.integers(3, 30)), s_rmin=2, s_rmax=max(3, side // 5),
                            n_cyl=int(rng.integers(0, 6)), seed=int(rng.integers(1, 1 << 30)))
        grid, offs, z = vo.synth_volume(spec)
        r = float(rng.choice([0.0, 1.5, 3.0, 5.25, 8.0, 12.0]))
        op = OPS[int(rng.integers(0, 4))]
        items.append((grid, offs, z, r, op))
    return items


@pytest.mark.parametrize("seed", [1, 2])
def test_batched_matches_oracle(ctx, vo, oracle, seed):
    items = _batch(vo, 12, seed)
    vols = [ctx.upload(g, o, z) for g, o, z, _, _ in items]
    outs, t = ctx.morph_batched(vols, [it[4] for it in items], [it[3] for it in items], "fast")
    assert t["kernel_launches"] > 0
    for (g, o, z, r, op), out in zip(items, outs):
        want = oracle.morph(ogrid(oracle, g), o, z, r, op)
        assert_same(ctx.download(out), want, tol=0.0, what=f"{g.nx}x{g.ny} {op} r={r}")


def test_batched_equals_single_calls(ctx, vo):
    items = _batch(vo, 6, 9)
    vols = [ctx.upload(g, o, z) for g, o, z, _, _ in items]
    outs, _ = ctx.morph_batched(vols, [it[4] for it in items], [it[3] for it in items], "fast")
    for v, (g, o, z, r, op), out in zip(vols, items, outs):
        single, _ = ctx.morph(v, op, r, "fast")
        a = ctx.download(out)
        b = ctx.download(single)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_batched_overflow_reruns(ctx, vo, oracle):
    # 40 thin plates in every column: each union outgrows the fixed 32-interval
    # slot, the spill region runs out, and the volume re-runs on its own
    nx, ny, k = 24, 20, 40
    base = np.arange(k, dtype=np.float64) * 3.0
    z = np.tile(np.stack([base, base + 1.0], 1).reshape(-1), nx * ny)
    offs = (np.arange(nx * ny + 1) * k).astype(np.int32)
    g = vo.Grid(nx, ny, (0, 0, 0), (nx, ny, 3 * k), 1.0, 0)
    g2, o2, z2 = vo.synth_volume(vo.SynthSpec(32, n_spheres=8, s_rmin=2, s_rmax=8, seed=5))
    vols = [ctx.upload(g, offs, z), ctx.upload(g2, o2, z2)]
    outs, t = ctx.morph_batched(vols, ["dilation", "closing"], [0.9, 3.0], "fast")
    assert t["overflow_columns"] >= 1  # the first volume re-ran through the single-volume path
    assert_same(ctx.download(outs[0]), oracle.morph(ogrid(oracle, g), offs, z, 0.9, "dilation"), tol=0.0)
    assert_same(ctx.download(outs[1]), oracle.morph(ogrid(oracle, g2), o2, z2, 3.0, "closing"), tol=0.0)


def test_plan_replays_identically(ctx, vo):
    items = _batch(vo, 8, 21)
    vols = [ctx.upload(g, o, z) for g, o, z, _, _ in items]
    b = ctx.batch(vols, [it[4] for it in items], [it[3] for it in items])
    st = b.stats()
    assert st["graph_nodes"] > 0 and st["graph_kernels"] > 0
    assert st["tile_rows"] in (1, 2, 4, 8)
    b.run()
    first = [ctx.download(o) for o in b.outputs()]
    t = b.run()
    assert t["pass2_ms"] > 0
    second = [ctx.download(o) for o in b.outputs()]
    for a, c in zip(first, second):
        assert np.array_equal(a[0], c[0]) and np.array_equal(a[1], c[1])
    # a second plan of the same shape reuses the autotuner's choice
    b2 = ctx.batch(vols, [it[4] for it in items], [it[3] for it in items])
    assert b2.stats()["tune_ms"] == [0.0, 0.0, 0.0, 0.0]
    assert b2.stats()["tile_rows"] == st["tile_rows"]


def test_plan_rejects_other_methods(ctx, vo):
    g, o, z = vo.synth_volume(vo.SynthSpec(32, n_spheres=4, s_rmin=2, s_rmax=6, seed=1))
    v = ctx.upload(g, o, z)
    with pytest.raises(vo.GpuError):
        ctx.batch([v], ["dilation"], [2.0], method="separable")


def test_batched_second_tier_without_rerun(ctx, vo, oracle):
    """A few columns with 40-interval unions: the second tier computes them and
    the spill region takes them, so no volume re-runs."""
    nx, ny, k = 64, 48, 40
    g0, o0, z0 = vo.synth_volume(vo.SynthSpec(64, n_spheres=30, s_rmin=2, s_rmax=8, seed=8, ny=48, zmax=200))
    cols = [z0[2 * o0[c]:2 * o0[c + 1]] for c in range(nx * ny)]
    base = 300.0 + np.arange(k) * 3.0
    plates = np.stack([base, base + 1.0], 1).reshape(-1)
    for y in range(10, 13):
        for x in range(20, 24):
            cols[x + nx * y] = np.concatenate([cols[x + nx * y], plates])
    offs = np.zeros(nx * ny + 1, np.int32)
    offs[1:] = np.cumsum([c.size // 2 for c in cols])
    z = np.concatenate(cols)
    g = vo.Grid(nx, ny, (0, 0, 0), (nx, ny, 500), 1.0, 0)
    v = ctx.upload(g, offs, z)
    outs, t = ctx.morph_batched([v], ["dilation"], [0.9], "fast")
    assert t["overflow_columns"] == 0
    assert_same(ctx.download(outs[0]), oracle.morph(ogrid(oracle, g), offs, z, 0.9, "dilation"), tol=0.0)


def test_plan_with_more_radii_than_the_table_cache(ctx, vo, oracle):
    """20 distinct radii in one plan: the context keeps at most 16 radius tables,
    so the plan must hold its own copies (every result checked)."""
    rng = np.random.default_rng(31)
    items = []
    for i in range(20):
        g, o, z = vo.synth_volume(vo.SynthSpec(24 + 2 * i, n_spheres=6, s_rmin=2, s_rmax=7, seed=100 + i))
        items.append((g, o, z, 1.0 + 0.5 * i, OPS[i % 4]))
    vols = [ctx.upload(g, o, z) for g, o, z, _, _ in items]
    b = ctx.batch(vols, [it[4] for it in items], [it[3] for it in items])
    for _ in range(2):
        # a later single call refills the context cache in between replays
        tmp, _ = ctx.morph(vols[0], "dilation", 40.25, "fast")
        tmp.free()
        b.run()
        for (g, o, z, r, op), out in zip(items, b.outputs()):
            assert_same(ctx.download(out), oracle.morph(ogrid(oracle, g), o, z, r, op), tol=0.0, what=f"{op} r={r}")


def test_batched_third_tier_without_rerun(ctx, vo, oracle):
    """A few columns with 150-interval unions: the FP64 third tier computes them
    inside the replay and the spill region takes them, so no volume re-runs."""
    nx, ny, k = 64, 48, 150
    g0, o0, z0 = vo.synth_volume(vo.SynthSpec(64, n_spheres=30, s_rmin=2, s_rmax=8, seed=8, ny=48, zmax=200))
    cols = [z0[2 * o0[c]:2 * o0[c + 1]] for c in range(nx * ny)]
    base = 300.0 + np.arange(k) * 3.0
    plates = np.stack([base, base + 1.0], 1).reshape(-1)
    for x in range(30, 36):
        cols[x + nx * 20] = np.concatenate([cols[x + nx * 20], plates])
    offs = np.zeros(nx * ny + 1, np.int32)
    offs[1:] = np.cumsum([c.size // 2 for c in cols])
    z = np.concatenate(cols)
    g = vo.Grid(nx, ny, (0, 0, 0), (nx, ny, 800), 1.0, 0)
    v = ctx.upload(g, offs, z)
    for op in ("dilation", "closing"):
        outs, t = ctx.morph_batched([v], [op], [0.9], "fast")
        assert t["overflow_columns"] == 0, op
        assert_same(ctx.download(outs[0]), oracle.morph(ogrid(oracle, g), offs, z, 0.9, op), tol=0.0, what=op)
