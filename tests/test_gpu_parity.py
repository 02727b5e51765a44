"""CUDA path vs the oracle, through the C ABI, on identical seeded inputs.

Separable (FP64) results must be bit-identical to the oracle (which is itself
pinned to the reference); the brute-force kernel must equal the oracle's
brute force; the two GPU methods agree within 1e-9 with identical topology.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN, assert_same, load_golden, ogrid

pytestmark = pytest.mark.gpu
OPS = ["dilation", "erosion", "opening", "closing"]


def run(ctx, grid, offs, z, op, r, method="separable"):
    v = ctx.upload(grid, offs, z)
    out, t = ctx.morph(v, op, r, method)
    res = ctx.download(out)
    assert t["kernel_launches"] > 0
    out.free()
    v.free()
    return res, t


METHODS = ["separable", "fast", "envelope"]


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: p.split("/")[-1][:-4])
@pytest.mark.parametrize("op", OPS)
@pytest.mark.parametrize("method", METHODS)
def test_gpu_matches_reference_golden(ctx, vo, path, op, method):
    grid, d = load_golden(path)
    got, _ = run(ctx, grid, d["offs"], d["z"], op, float(d["radius"]), method)
    assert_same(got, (d[f"{op}_offs"], d[f"{op}_z"]), tol=1e-9, what=f"{path}:{op}")


CASES = [
    dict(n=96, n_spheres=60, s_rmin=4, s_rmax=24, seed=21),
    dict(n=128, n_cyl=80, c_rmin=1, c_rmax=4, seed=22),
    dict(n=112, n_spheres=90, sphere_dist="lognormal", s_median=8, s_sigma=0.5, s_rmin=2, s_rmax=40, n_cyl=30,
         seed=23),
]
RADII = [0.0, 1.0, 4.5, 8.0, 16.0, 32.0]


@pytest.mark.parametrize("case", range(len(CASES)))
@pytest.mark.parametrize("r", RADII)
@pytest.mark.parametrize("method", METHODS)
def test_gpu_dilation_bit_exact(ctx, vo, oracle, case, r, method):
    grid, offs, z = vo.synth_volume(vo.SynthSpec(**CASES[case]))
    want = oracle.morph(ogrid(oracle, grid), offs, z, r, "dilation")
    got, _ = run(ctx, grid, offs, z, "dilation", r, method)
    assert_same(got, want, tol=0.0, what=f"case {case} r={r}")


@pytest.mark.parametrize("case", range(len(CASES)))
@pytest.mark.parametrize("op", ["erosion", "opening", "closing"])
@pytest.mark.parametrize("method", METHODS)
def test_gpu_chained_ops_bit_exact(ctx, vo, oracle, case, op, method):
    grid, offs, z = vo.synth_volume(vo.SynthSpec(**CASES[case]))
    want = oracle.morph(ogrid(oracle, grid), offs, z, 6.0, op)
    got, _ = run(ctx, grid, offs, z, op, 6.0, method)
    assert_same(got, want, tol=0.0, what=f"case {case} {op}")


@pytest.mark.parametrize("r", [3.0, 7.5])
def test_gpu_brute_force(ctx, vo, oracle, r):
    grid, offs, z = vo.synth_volume(vo.SynthSpec(64, n_spheres=30, s_rmin=3, s_rmax=16, n_cyl=10, seed=31))
    want = oracle.morph(ogrid(oracle, grid), offs, z, r, "dilation", "brute")
    got, _ = run(ctx, grid, offs, z, "dilation", r, "brute")
    assert_same(got, want, tol=0.0, what="brute")
    sep, _ = run(ctx, grid, offs, z, "dilation", r, "separable")
    assert_same(got, sep, tol=1e-9, what="brute vs separable")


@pytest.mark.parametrize("method", METHODS)
def test_gpu_edge_shapes(ctx, vo, oracle, method):
    rng = np.random.default_rng(5)
    for nx, ny in [(1, 1), (1, 37), (41, 1), (3, 70), (33, 5)]:
        counts = rng.integers(0, 4, size=nx * ny)
        offs = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
        z = []
        for c in counts:
            v = np.sort(rng.uniform(0, 50, size=2 * c))
            z.extend(v)
        z = np.array(z, dtype=np.float64)
        grid = vo.Grid(nx, ny, (0, 0, 0), (nx, ny, 50), 1.0, 0)
        for op in OPS:
            want = oracle.morph(ogrid(oracle, grid), offs, z, 3.5, op)
            got, _ = run(ctx, grid, offs, z, op, 3.5, method)
            assert_same(got, want, tol=0.0, what=f"{nx}x{ny} {op}")


@pytest.mark.parametrize("method", METHODS)
def test_gpu_empty_and_full_columns(ctx, vo, oracle, method):
    nx, ny = 20, 17
    counts = np.zeros(nx * ny, np.int64)
    counts[::7] = 1
    offs = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
    z = np.tile([0.0, 30.0], int(counts.sum()))  # full-height columns (clipped at both ends)
    grid = vo.Grid(nx, ny, (0, 0, 0), (nx, ny, 30), 1.0, 0)
    for op in OPS:
        want = oracle.morph(ogrid(oracle, grid), offs, z, 2.5, op)
        got, _ = run(ctx, grid, offs, z, op, 2.5, method)
        assert_same(got, want, tol=0.0, what=op)
    empty = np.zeros(nx * ny + 1, np.int32)
    got, _ = run(ctx, grid, empty, np.zeros(0), "dilation", 4.0, method)
    assert got[0][-1] == 0


@pytest.mark.parametrize("method", METHODS)
def test_gpu_zero_length_and_touching_segments(ctx, vo, oracle, method):
    nx, ny = 24, 24
    rng = np.random.default_rng(8)
    offs = [0]
    z = []
    for c in range(nx * ny):
        k = int(rng.integers(0, 3))
        pts = np.sort(rng.choice(np.arange(0, 40, 0.5), size=2 * k, replace=False))
        if k and rng.random() < 0.3:
            pts[1] = pts[0]  # a point segment
        z.extend(pts)
        offs.append(offs[-1] + k)
    offs = np.array(offs, np.int32)
    z = np.array(z, np.float64)
    grid = vo.Grid(nx, ny, (0, 0, 0), (nx, ny, 40), 1.0, 0)
    for r in [0.0, 1.0, 2.0, 5.0]:  # exact lattice radii produce many exact touches
        want = oracle.morph(ogrid(oracle, grid), offs, z, r, "dilation")
        got, _ = run(ctx, grid, offs, z, "dilation", r, method)
        assert_same(got, want, tol=0.0, what=f"r={r}")


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("k", [40, 63, 64, 100, 127, 128, 150])
def test_gpu_overflow_path(ctx, vo, oracle, method, k):
    # k thin disjoint plates per column dilated by r = 0.9 give exactly k
    # union intervals, overflowing the kernels' working lists at known sizes
    # (FP32 method: its 64-slot variant for dense inputs holds 63 intervals
    # beside its sentinel, the 128-slot second tier 127, beyond that the
    # FP64 list); every tier must give the same answer
    nx, ny = 40, 40
    base = np.arange(k, dtype=np.float64) * 3.0
    z = np.stack([base, base + 1.0], 1).reshape(-1)
    offs = (np.arange(nx * ny + 1) * k).astype(np.int32)
    zz = np.tile(z, nx * ny)
    grid = vo.Grid(nx, ny, (0, 0, 0), (nx, ny, 3 * k), 1.0, 0)
    want = oracle.morph(ogrid(oracle, grid), offs, zz, 0.9, "dilation")
    got, t = run(ctx, grid, offs, zz, "dilation", 0.9, method)
    if method == "fast":
        assert (t["overflow_columns"] > 0) == (k > 63), t["overflow_columns"]
    elif method == "envelope":
        # 64 intervals fit its output slots; beyond, the volume takes the painter form, which re-runs
        assert (t["overflow_columns"] > 0) == (k > 64), t["overflow_columns"]
    else:
        assert t["overflow_columns"] > 0
    assert_same(got, want, tol=0.0)


def test_gpu_rejects_bad_input(ctx, vo):
    # 40 columns wide: x_s + r rounds up to the next integer for x_s >= 7
    grid = vo.Grid(40, 40, (0, 0, 0), (40, 40, 40), 1.0, 0)
    offs = np.zeros(1601, np.int32)
    v = ctx.upload(grid, offs, np.zeros(0))
    with pytest.raises(vo.GpuError) as e:
        ctx.morph(v, "dilation", -1.0)
    assert e.value.code == vo.VO_EINVAL
    with pytest.raises(vo.GpuError) as e:
        ctx.morph(v, "dilation", 3.0 - 1e-15)  # a hair below a lattice distance
    assert e.value.code == vo.VO_ERADIUS
    bad = offs.copy()
    bad[3] = 5  # offsets must not decrease
    with pytest.raises(vo.GpuError):
        ctx.upload(grid, bad, np.zeros(10))
    import ctypes as C
    out_h = C.c_void_p()
    rc = vo.lib().vo_morph(ctx.handle, 0, 99, 2.0, v.handle, C.byref(out_h), None)  # unknown method
    assert rc == vo.VO_EINVAL and not out_h.value
    rc = vo.lib().vo_morph(ctx.handle, 7, 0, 2.0, v.handle, C.byref(out_h), None)  # unknown op
    assert rc == vo.VO_EINVAL
    # the context stays usable after errors
    out, _ = ctx.morph(v, "dilation", 2.0)
    assert out.nseg == 0


def test_gpu_xor_volume(ctx, vo, oracle):
    grid, offs, z = vo.synth_volume(vo.SynthSpec(64, n_spheres=30, s_rmin=3, s_rmax=16, seed=41))
    a = ctx.upload(grid, offs, z)
    assert ctx.xor_volume(a, a) == 0.0
    e, _ = ctx.morph(a, "erosion", 3.0)
    eo, ez = ctx.download(e)
    want = oracle.xor_volume(ogrid(oracle, grid), (offs, z), (eo, ez))
    got = ctx.xor_volume(a, e)
    assert got == pytest.approx(want, rel=1e-12)


def test_gpu_measure_matches_oracle(ctx, vo, oracle):
    """numSegments / get_volume (CompressedVolume.cpp:61-83) on the device; the volume is a sum in a
    different order from the reference's sequential one, so it agrees to rounding."""
    grid, offs, z = vo.synth_volume(vo.SynthSpec(80, ny=70, n_spheres=40, s_rmin=2, s_rmax=15, n_cyl=6, seed=44))
    g2 = vo.Grid(grid.nx, grid.ny, grid.origin, grid.extent, 0.25, 0)  # spacing enters as spacing^3
    for g in (grid, g2):
        v = ctx.upload(g, offs, z)
        n, vol = ctx.measure(v)
        assert n == int(offs[-1])
        assert vol == pytest.approx(oracle.get_volume(ogrid(oracle, g), offs, z), rel=1e-12)
        v.free()
    empty = ctx.upload(grid, np.zeros(grid.ncols + 1, np.int32), np.zeros(0))
    assert ctx.measure(empty) == (0, 0.0)


def test_gpu_dexelize_matches_oracle(ctx, vo, oracle):
    verts, tris = vo.synth_torus(256, 64, 0.30, 0.10, 0.01, seed=1)
    og, offs, z = oracle.dexelize(verts, tris, num_dexels=128, padding=10)
    v = ctx.dexelize(verts, tris, num_dexels=128, padding=10)
    assert (v.grid.nx, v.grid.ny) == (og.nx, og.ny)
    assert v.grid.spacing == og.spacing and tuple(v.grid.origin) == tuple(og.origin)
    got = ctx.download(v)
    assert_same(got, (offs, z), tol=0.0, what="dexelize")
    assert np.all(np.diff(offs) >= 0) and got[0][-1] > 0


@pytest.mark.parametrize("method", METHODS + ["brute"])
def test_gpu_inverted_pairs_normalised(ctx, vo, oracle, method):
    # columns holding inverted pairs (what negate_ray leaves when values exceed
    # the complement range) behave as their two endpoints
    rng = np.random.default_rng(12)
    nx, ny = 30, 26
    offs = [0]
    z = []
    for c in range(nx * ny):
        k = int(rng.integers(0, 4))
        v = np.sort(rng.uniform(0, 40, size=2 * k))
        pairs = v.reshape(-1, 2).tolist()
        if pairs and rng.random() < 0.4:
            a, b = pairs[0]
            pairs[0] = [b + 0.5, a]  # inverted
        for a, b in pairs:
            z += [a, b]
        offs.append(offs[-1] + len(pairs))
    offs = np.array(offs, np.int32)
    z = np.array(z, np.float64)
    grid = vo.Grid(nx, ny, (0, 0, 0), (nx, ny, 40), 1.0, 0)
    for r in [2.0, 4.5]:
        want = oracle.morph(ogrid(oracle, grid), offs, z, r, "dilation", "brute" if method == "brute" else "separable")
        got, _ = run(ctx, grid, offs, z, "dilation", r, method)
        assert_same(got, want, tol=0.0, what=f"{method} r={r}")


@pytest.mark.parametrize("shift", [-3.0e5, 7.5e5])
def test_gpu_fast_far_from_origin(ctx, vo, oracle, shift):
    """z values of magnitude ~1e5-1e6 leave FP32 about 0.06 dexel of precision:
    most merge decisions fall inside the guard band and are taken in FP64, and
    the result stays bit-identical (both methods, all ops)."""
    grid, offs, z = vo.synth_volume(vo.SynthSpec(40, n_spheres=12, s_rmin=2, s_rmax=9, n_cyl=3, seed=17))
    z = z + shift
    g = vo.Grid(grid.nx, grid.ny, (0.0, 0.0, shift), grid.extent, grid.spacing, grid.padding)
    for op in ("dilation", "erosion", "closing"):
        want = oracle.morph(ogrid(oracle, g), offs, z, 5.5, op)
        got, _ = run(ctx, g, offs, z, op, 5.5, "fast")
        assert_same(got, want, tol=0.0, what=f"{op} shift={shift}")


def test_gpu_fast_largest_radius(ctx, vo, oracle):
    """r = 255 (the largest radius; ~51,000 (|dx|, |dy|) pairs) on a small grid."""
    grid, offs, z = vo.synth_volume(vo.SynthSpec(48, n_spheres=10, s_rmin=2, s_rmax=8, seed=23))
    want = oracle.morph(ogrid(oracle, grid), offs, z, 255.0, "dilation")
    got, _ = run(ctx, grid, offs, z, "dilation", 255.0, "fast")
    assert_same(got, want, tol=0.0)
    outs, _ = ctx.morph_batched([ctx.upload(grid, offs, z)], ["dilation"], [255.0], "fast")
    assert_same(ctx.download(outs[0]), want, tol=0.0, what="batch plan")


@pytest.mark.parametrize("shape", [(1, 200), (200, 1), (3, 97)])
def test_gpu_fast_thin_grids_batch(ctx, vo, oracle, shape):
    """Grids one or a few columns wide, through a batch plan with every op."""
    nx, ny = shape
    rng = np.random.default_rng(nx * 1000 + ny)
    cols = []
    for _ in range(nx * ny):
        k = int(rng.integers(0, 4))
        v = np.sort(rng.uniform(0, 60, 2 * k))
        cols.append(v)
    offs = np.zeros(nx * ny + 1, np.int32)
    offs[1:] = np.cumsum([c.size // 2 for c in cols])
    z = np.concatenate(cols) if offs[-1] else np.zeros(0)
    g = vo.Grid(nx, ny, (0, 0, 0), (nx, ny, 60), 1.0, 0)
    v = ctx.upload(g, offs, z)
    ops = ["dilation", "erosion", "opening", "closing"]
    outs, _ = ctx.morph_batched([v] * 4, ops, [3.5] * 4, "fast")
    for op, out in zip(ops, outs):
        assert_same(ctx.download(out), oracle.morph(ogrid(oracle, g), offs, z, 3.5, op), tol=0.0, what=op)
