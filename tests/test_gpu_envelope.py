"""The envelope form of the separable method (VO_METHOD_ENVELOPE) beyond the
parity suites it shares with the other methods: volumes split into several
bands of rows, lines and rows whose sweep state outgrows shared memory (the
re-runs with global-memory state), and the full-size workloads."""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import assert_same, ogrid

pytestmark = pytest.mark.gpu


def run(ctx, grid, offs, z, op, r, method="envelope"):
    v = ctx.upload(grid, offs, z)
    out, t = ctx.morph(v, op, r, method)
    res = ctx.download(out)
    out.free()
    v.free()
    return res, t


@pytest.mark.parametrize("cap", [5000, 40000])
def test_envelope_in_bands(ctx, vo, oracle, cap, monkeypatch):
    """A cap on the pass-1 intermediate splits the rows into bands; each band
    re-sweeps its lines from floor(r) rows before it, and the result is unchanged."""
    grid, offs, z = vo.synth_volume(vo.SynthSpec(96, ny=80, n_spheres=40, s_rmin=2, s_rmax=14, n_cyl=8, seed=91))
    monkeypatch.setenv("VO_ENVELOPE_BAND_PIECES", str(cap))
    for op, r in (("dilation", 7.5), ("closing", 4.0)):
        got, t = run(ctx, grid, offs, z, op, r)
        assert_same(got, oracle.morph(ogrid(oracle, grid), offs, z, r, op), tol=0.0, what=f"{op} cap={cap}")


def test_envelope_states_beyond_shared_memory(ctx, vo, oracle):
    """150 thin plates per column, shifted from row to row and column to column:
    the pass-1 envelope of a line holds thousands of slivers and the pass-2 row
    state several thousand stadiums, beyond both shared-memory capacities, so
    both sweeps re-run those lines and rows with global-memory state."""
    nx, ny, k = 24, 20, 150
    offs = (np.arange(nx * ny + 1) * k).astype(np.int32)
    z = []
    for y in range(ny):
        for x in range(nx):
            s = 0.11 * (y % 7) + 0.05 * (x % 5)
            base = np.arange(k) * 3.0 + s
            z.append(np.stack([base, base + 0.5], 1).reshape(-1))
    z = np.concatenate(z)
    grid = vo.Grid(nx, ny, (0, 0, 0), (nx, ny, 3 * k + 1), 1.0, 0)
    got, t = run(ctx, grid, offs, z, "dilation", 4.0)
    assert_same(got, oracle.morph(ogrid(oracle, grid), offs, z, 4.0, "dilation"), tol=0.0)
    assert t["mid_pieces"] > 0  # the envelope kernels ran (the painter form reports its own pieces)
    assert t["overflow_columns"] > 0  # lines or rows re-ran with global-memory state


@pytest.mark.parametrize("cap", [48, 160])
def test_envelope_rows_rerun_in_global_memory(ctx, vo, oracle, cap, monkeypatch):
    """A lowered first-tier stadium capacity (VO_ENVELOPE_STATE_CAP) sends rows
    of an ordinary volume to the re-run with global-memory state, which prunes
    dominated stadiums the same way: results unchanged, re-runs counted."""
    grid, offs, z = vo.synth_volume(vo.SynthSpec(80, ny=72, n_spheres=60, s_rmin=2, s_rmax=16, n_cyl=10, seed=93))
    monkeypatch.setenv("VO_ENVELOPE_STATE_CAP", str(cap))
    reruns = 0
    for op, r in (("dilation", 9.0), ("erosion", 5.5), ("closing", 12.0)):
        got, t = run(ctx, grid, offs, z, op, r)
        reruns += t["overflow_columns"]
        assert_same(got, oracle.morph(ogrid(oracle, grid), offs, z, r, op), tol=0.0, what=f"{op} cap={cap}")
    assert reruns > 0


def test_envelope_global_sweep_in_row_chunks(ctx, vo, oracle, monkeypatch):
    """The global-memory sweep launched over a few rows at a time
    (VO_ENVELOPE_ROW_CHUNK), every row sent there (VO_ENVELOPE_STATE_CAP):
    results unchanged."""
    grid, offs, z = vo.synth_volume(vo.SynthSpec(72, ny=45, n_spheres=50, s_rmin=2, s_rmax=12, n_cyl=6, seed=95))
    monkeypatch.setenv("VO_ENVELOPE_STATE_CAP", "16")
    monkeypatch.setenv("VO_ENVELOPE_ROW_CHUNK", "7")
    for op, r in (("dilation", 6.5), ("opening", 4.0)):
        got, t = run(ctx, grid, offs, z, op, r)
        assert t["overflow_columns"] > 0
        assert_same(got, oracle.morph(ogrid(oracle, grid), offs, z, r, op), tol=0.0, what=op)


def test_envelope_pruning_keeps_nested_plates(ctx, vo, oracle):
    """Columns whose segments nest inside their neighbours' with margins just
    above and just below what the chord growth allows: stadiums that a newer
    piece holds for the rest of their lives leave the state, the others stay,
    and the union equals the oracle's."""
    nx, ny = 40, 12
    rng = np.random.default_rng(7)
    cols = []
    for y in range(ny):
        for x in range(nx):
            base = 50.0 + 0.37 * ((x * 7 + y * 3) % 11)
            w = 3.0 + 0.5 * np.sin(0.7 * x + 0.3 * y)
            eps = rng.choice([-1e-9, 0.0, 1e-9, 0.25])
            cols.append([base - eps, base + w + eps, base + w + 4.0, base + w + 4.0 + 0.5 * (x % 3)])
    offs = (np.arange(nx * ny + 1) * 2).astype(np.int32)
    z = np.asarray(cols, dtype=np.float64).reshape(-1)
    grid = vo.Grid(nx, ny, (0, 0, 0), (nx, ny, 80), 1.0, 0)
    for r in (3.0, 6.5, 11.0):
        got, t = run(ctx, grid, offs, z, "dilation", r)
        assert t["mid_pieces"] > 0
        assert_same(got, oracle.morph(ogrid(oracle, grid), offs, z, r, "dilation"), tol=0.0, what=f"r={r}")


@pytest.fixture(scope="module")
def spheres_cyl2048(vo):
    return vo.workload("spheres_cyl2048", seed=1)


@pytest.mark.parametrize("r", [32.0, 64.0])
def test_envelope_fullsize_equals_fast(ctx, vo, spheres_cyl2048, r):
    """2048^2 spheres + cylinders: the FP64 envelope sweeps and the FP32-guarded
    kernel (bit-exact against the oracle on sampled columns in
    test_gpu_fullsize) give identical volumes."""
    grid, offs, z = spheres_cyl2048
    v = ctx.upload(grid, offs, z)
    a, ta = ctx.morph(v, "dilation", r, "envelope")
    b, _ = ctx.morph(v, "dilation", r, "fast")
    ao, az = ctx.download(a)
    bo, bz = ctx.download(b)
    assert np.array_equal(ao, bo) and np.array_equal(az, bz)
    assert ta["mid_pieces"] > 0
    a.free()
    b.free()
    v.free()
