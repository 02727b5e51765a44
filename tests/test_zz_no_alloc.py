"""The allocation-free xor volume entry point (vo_xor_volume_noalloc).

It exists for callers that must not allocate device memory while they run
(code inside a stream host callback, services whose device memory belongs to
another allocator, hot loops kept off the allocator); its scratch is a fixed
device array shared by all calls. These tests call it through the C ABI twice
in a row, on different inputs, and check each result against the allocating
entry point vo_xor_volume. The file sorts last so that a run stopping at the
first failure has already run every other test.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_xor_matches_allocating_entry_point_twice(ctx, vo):
    grid, offs, z = vo.synth_volume(vo.SynthSpec(96, n_spheres=50, s_rmin=3, s_rmax=20, n_cyl=10, seed=77))
    a = ctx.upload(grid, offs, z)
    b, _ = ctx.morph(a, "erosion", 3.0, "fast")
    c, _ = ctx.morph(a, "erosion", 6.0, "fast")
    g = grid.to_c()
    pa = a.device_ptrs()
    results = []
    for other in (b, c):
        want = ctx.xor_volume(a, other)
        po = other.device_ptrs()
        got = C.c_double(-1.0)
        rc = vo.lib().vo_xor_volume_noalloc(C.byref(g), pa[0], pa[1], po[0], po[1], ctx.stream, C.byref(got))
        assert rc == vo.VO_OK
        assert got.value == pytest.approx(want, rel=1e-12)
        results.append(got.value)
    assert results[0] != results[1]  # the second call did not reuse the first call's partial sums


def test_noalloc_rejects_grids_beyond_its_scratch(vo):
    g = vo.Grid(8192, 4096, (0, 0, 0), (8192, 4096, 10), 1.0, 0).to_c()  # 33.5M columns > 16.8M
    out = C.c_double(-1.0)
    fake = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = vo.lib().vo_xor_volume_noalloc(C.byref(g), fake, fake, fake, fake, None, C.byref(out))
    assert rc == vo.VO_ERANGE and out.value == -1.0
