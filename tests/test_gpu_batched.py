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
    # 60 thin plates per column: more union intervals than a slot holds
    nx, ny, k = 24, 20, 60
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
