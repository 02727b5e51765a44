"""Asynchronous copies (vo_volume_upload_async / vo_volume_download_async): the
copies run on the context's copy stream and overlap its kernels; every entry
point that reads an uploaded volume waits for its copy, and freeing a volume
waits for its download. Results must equal the synchronous path's bit for bit."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import ogrid

pytestmark = pytest.mark.gpu


def pinned(a, dtype):
    import torch

    t = torch.empty(max(a.size, 2), dtype={np.int32: torch.int32, np.float64: torch.float64}[dtype],
                    pin_memory=True)
    v = t.numpy()
    v[:a.size] = a
    return t, v[:a.size] if a.size else v[:2]


def volumes(vo, n):
    out = []
    for i in range(n):
        g, o, z = vo.synth_volume(vo.SynthSpec(40 + 8 * i, ny=36, n_spheres=20 + 5 * i, s_rmin=2, s_rmax=9, n_cyl=3,
                                               seed=120 + i))
        out.append((g, np.ascontiguousarray(o, np.int32), np.ascontiguousarray(z, np.float64)))
    return out


def test_async_round_trip_equals_sync(ctx, vo, oracle):
    g, o, z = volumes(vo, 1)[0]
    keep = []
    to, po = pinned(o, np.int32)
    tz, pz = pinned(z, np.float64)
    keep += [to, tz]
    v = ctx.upload_async(g, po, pz)
    out, _ = ctx.morph(v, "closing", 5.5, "fast")
    ta, ho = pinned(np.zeros(g.ncols + 1, np.int32), np.int32)
    tb, hz = pinned(np.zeros(2 * out.nseg, np.float64), np.float64)
    n_o, n_z = ctx.download_async(out, ho, hz)
    ctx.sync()
    ro, rz = oracle.morph(ogrid(oracle, g), o, z, 5.5, "closing")
    assert np.array_equal(ho[:n_o], ro) and np.array_equal(hz[:n_z], rz)
    out.free()
    v.free()


def test_pipelined_steps(ctx, vo):
    """Upload of step i + 1 issued before the dilation of step i, download of
    step i after it, output freed right after its download was queued: every
    result equals the synchronous path's."""
    items = volumes(vo, 5)
    keep, ins = [], []
    for g, o, z in items:
        to, po = pinned(o, np.int32)
        tz, pz = pinned(z, np.float64)
        keep += [to, tz]
        ins.append((g, po, pz))
    results = []
    nxt = ctx.upload_async(*ins[0])
    for i in range(len(ins)):
        cur = nxt
        if i + 1 < len(ins):
            nxt = ctx.upload_async(*ins[i + 1])
        outs, _ = ctx.morph_batched([cur], ["dilation"], [4.0 + i], "fast")
        o = outs[0]
        tb1, ho = pinned(np.zeros(items[i][0].ncols + 1, np.int32), np.int32)
        tb2, hz = pinned(np.zeros(max(2 * o.nseg, 2), np.float64), np.float64)
        keep += [tb1, tb2]
        n = ctx.download_async(o, ho, hz)
        results.append((ho, hz, n))
        o.free()    # waits for its download in stream order
        cur.free()
    ctx.sync()
    for (g, po, pz), (ho, hz, (n_o, n_z)), i in zip(ins, results, range(len(ins))):
        v = ctx.upload(g, np.array(po), np.array(pz))
        ref, _ = ctx.morph(v, "dilation", 4.0 + i, "fast")
        ro, rz = ctx.download(ref)
        assert np.array_equal(ho[:n_o], ro) and np.array_equal(hz[:n_z], rz), f"step {i}"
        ref.free()
        v.free()


def test_async_inputs_to_plans_and_reductions(ctx, vo):
    """A batch plan, the xor and measure reductions read async-uploaded volumes;
    a volume freed without any use waits for its copy."""
    (g, o, z), = volumes(vo, 1)
    to, po = pinned(o, np.int32)
    tz, pz = pinned(z, np.float64)
    a = ctx.upload_async(g, po, pz)
    b = ctx.upload_async(g, po, pz)
    unused = ctx.upload_async(g, po, pz)
    unused.free()
    plan = ctx.batch([a], ["dilation"], [3.5], "fast")
    plan.run()
    (pa,) = plan.outputs()
    ref, _ = ctx.morph(b, "dilation", 3.5, "fast")
    assert ctx.xor_volume(pa, ref) == 0.0
    assert ctx.measure(a) == ctx.measure(b)
    n, vol = ctx.measure(b)
    assert n == len(z) // 2
    plan.free()  # before its inputs
    for v in (pa, ref, a, b):
        v.free()
    ctx.sync()
    del to, tz


@pytest.mark.parametrize("where", [5, 700_000, 1_099_998])
def test_uploads_reject_decreasing_offsets_on_large_grids(ctx, vo, where):
    """Grids of more than 2^20 columns are checked by several host threads: a
    decrease anywhere (first, middle or last chunk) is refused by both uploads."""
    g = vo.Grid(1100, 1000, (0, 0, 0), (1100, 1000, 10), 1.0, 0)
    offs = np.arange(g.ncols + 1, dtype=np.int32) // 4
    z = np.tile(np.array([1.0, 2.0]), int(offs[-1]))
    to, po = pinned(offs, np.int32)
    tz, pz = pinned(z, np.float64)
    good = ctx.upload_async(g, po, pz)
    good.free()
    po[where] = po[where + 1] + 1
    with pytest.raises(vo.GpuError):
        ctx.upload(g, np.array(po), z)
    with pytest.raises(vo.GpuError):
        ctx.upload_async(g, po, pz)
    ctx.sync()
    del to, tz


def test_async_round_trip_in_pieces(ctx, vo):
    """More segments than one 64 MB copy piece (4,194,304): uploaded and
    downloaded asynchronously in several pieces, the volume comes back bit for
    bit, and a dilation of it equals the synchronous path's."""
    g = vo.Grid(2048, 1024, (0, 0, 0), (2048, 1024, 64), 1.0, 0)
    rng = np.random.default_rng(5)
    offs = (np.arange(g.ncols + 1, dtype=np.int64) * 3).astype(np.int32)  # 6.3 M segments
    base = np.sort(rng.uniform(0.0, 60.0, (g.ncols, 6)), axis=1)
    z = np.ascontiguousarray(base.reshape(-1))
    to, po = pinned(offs, np.int32)
    tz, pz = pinned(z, np.float64)
    v = ctx.upload_async(g, po, pz)
    tb1, ho = pinned(np.zeros(g.ncols + 1, np.int32), np.int32)
    tb2, hz = pinned(np.zeros(z.size, np.float64), np.float64)
    ctx.download_async(v, ho, hz)
    ctx.sync()
    assert np.array_equal(ho, offs) and np.array_equal(hz, z)
    out, _ = ctx.morph(v, "dilation", 2.0, "fast")
    ta, ro = pinned(np.zeros(g.ncols + 1, np.int32), np.int32)
    tb, rz = pinned(np.zeros(2 * out.nseg, np.float64), np.float64)
    n_o, n_z = ctx.download_async(out, ro, rz)
    ctx.sync()
    ref_o, ref_z = ctx.download(out)
    assert np.array_equal(ro[:n_o], ref_o) and np.array_equal(rz[:n_z], ref_z)
    out.free()
    v.free()
