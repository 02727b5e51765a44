"""The allocation-free xor volume entry point (vo_xor_volume_noalloc).

It exists for callers that must not allocate device memory while they run:
services whose device memory belongs to another allocator, and hot loops kept
off the allocator. Its scratch is a fixed device array shared by all calls.
These tests call it through the C ABI twice in a row, on different inputs, and
check each result against the allocating entry point vo_xor_volume, on a grid
whose column count is a multiple of the reduction's 256-column blocks, on one
that is not, and on the largest grids the scratch accepts. The file sorts last
so that a run stopping at the first failure has already run every other test.
"""
from __future__ import annotations

import ctypes as C

import pytest

pytestmark = pytest.mark.gpu


def _noalloc(vo, ctx, grid, a, b):
    g = grid.to_c()
    pa, pb = a.device_ptrs(), b.device_ptrs()
    got = C.c_double(-1.0)
    rc = vo.lib().vo_xor_volume_noalloc(C.byref(g), pa[0], pa[1], pb[0], pb[1], ctx.stream, C.byref(got))
    assert rc == vo.VO_OK
    return got.value


@pytest.mark.parametrize("nx,ny", [(96, 96), (97, 95)])
def test_noalloc_xor_matches_allocating_entry_point_twice(ctx, vo, nx, ny):
    grid, offs, z = vo.synth_volume(vo.SynthSpec(nx, ny=ny, n_spheres=50, s_rmin=3, s_rmax=20, n_cyl=10, seed=77))
    a = ctx.upload(grid, offs, z)
    b, _ = ctx.morph(a, "erosion", 3.0, "fast")
    c, _ = ctx.morph(a, "erosion", 6.0, "fast")
    results = []
    for other in (b, c):
        want = ctx.xor_volume(a, other)
        got = _noalloc(vo, ctx, grid, a, other)
        assert got == pytest.approx(want, rel=1e-12)
        results.append(got)
    assert results[0] != results[1]  # the second call did not reuse the first call's partial sums
    for v in (a, b, c):
        v.free()


@pytest.mark.parametrize("nx,ny", [(4096, 4096), (4095, 4097)])
def test_noalloc_xor_at_the_largest_grids(ctx, vo, nx, ny):
    # 16,777,216 columns fill every partial-sum slot; 16,777,215 leave the last block one column short
    ga, oa, za = vo.synth_volume(vo.SynthSpec(nx, ny=ny, zmax=64, n_spheres=40, s_rmin=4, s_rmax=30, seed=5))
    _, ob, zb = vo.synth_volume(vo.SynthSpec(nx, ny=ny, zmax=64, n_spheres=40, s_rmin=4, s_rmax=30, seed=6))
    a = ctx.upload(ga, oa, za)
    b = ctx.upload(ga, ob, zb)
    for _ in range(2):
        want = ctx.xor_volume(a, b)
        assert want > 0
        assert _noalloc(vo, ctx, ga, a, b) == pytest.approx(want, rel=1e-12)
    a.free()
    b.free()


def test_noalloc_rejects_grids_beyond_its_scratch(vo):
    g = vo.Grid(8192, 4096, (0, 0, 0), (8192, 4096, 10), 1.0, 0).to_c()  # 33.5M columns > 16.8M
    out = C.c_double(-1.0)
    fake = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = vo.lib().vo_xor_volume_noalloc(C.byref(g), fake, fake, fake, fake, None, C.byref(out))
    assert rc == vo.VO_ERANGE and out.value == -1.0


def test_noalloc_rejects_null_value_arrays(vo):
    g = vo.Grid(8, 8, (0, 0, 0), (8, 8, 10), 1.0, 0).to_c()
    out = C.c_double(-1.0)
    fake = C.c_void_p(16)  # never dereferenced: the argument checks come first
    rc = vo.lib().vo_xor_volume_noalloc(C.byref(g), fake, None, fake, fake, None, C.byref(out))
    assert rc == vo.VO_EINVAL and out.value == -1.0
