"""The 2D path: pixel images of the reference's CompressedImage (src/vor2d,
CompressedImage.cpp:608-647) dilated, eroded, opened and closed.

* the oracle restatement against fixtures written by the reference's own 2D
  core (compiled unmodified; tests/golden/2d/) and, where its sources exist,
  against that build on seeded random images;
* the GPU (vo_image_morph, through the C ABI) against the fixtures and the
  oracle, bit for bit (integer pixel spans), including one-pixel-wide and
  one-row images, empty and full rows, integer radii and radius 0, and its
  argument checks;
* the FP64 twin (DoubleCompressedImage, DoubleCompressedImage.cpp:680-720) the
  same way: oracle against fixtures written by the reference's own build and
  against that build; vo_image_morph_f64 against both, bit for bit."""
from __future__ import annotations

import ctypes as C
import glob
import os

import numpy as np
import pytest

from conftest import ROOT
from imageutil import blobs, from_mask, random_f64

GOLDEN2D = sorted(p for p in glob.glob(os.path.join(ROOT, "tests", "golden", "2d", "*.npz"))
                  if not os.path.basename(p).startswith("f64_"))
GOLDEN2D_F64 = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "2d", "f64_*.npz")))
OPS = {"dilation": "dilate", "erosion": "erode", "opening": "open", "closing": "close"}


@pytest.mark.parametrize("path", GOLDEN2D, ids=lambda p: os.path.basename(p)[:-4])
@pytest.mark.parametrize("op", list(OPS))
def test_oracle_image_matches_reference_fixture(oracle, path, op):
    d = np.load(path)
    got = oracle.image_morph(int(d["width"]), int(d["height"]), d["offs"], d["events"], float(d["radius"]), OPS[op])
    assert np.array_equal(got[0], d[f"{op}_offs"]) and np.array_equal(got[1], d[f"{op}_events"])


def test_oracle_image_matches_reference_build(oracle):
    if not oracle.ref2d_available():
        pytest.skip("reference sources absent: pinned by the fixtures instead")
    rng = np.random.default_rng(3)
    for trial in range(40):
        w, h = int(rng.integers(1, 70)), int(rng.integers(1, 70))
        r = float(rng.choice([0.0, 0.7, 1.0, 2.0, 3.3, 5.0, 8.5, 12.0]))
        offs, ev = blobs(w, h, int(rng.integers(0, 25)), int(rng.integers(1, 1 << 30)), rmax=10,
                         noise=float(rng.choice([0.0, 0.05, 0.3])))
        for op in OPS.values():
            a = oracle.image_morph(w, h, offs, ev, r, op)
            b = oracle.ref_image_morph(w, h, offs, ev, r, op)
            assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), (trial, w, h, r, op)


@pytest.mark.gpu
@pytest.mark.parametrize("path", GOLDEN2D, ids=lambda p: os.path.basename(p)[:-4])
def test_gpu_image_matches_reference_fixture(ctx, path):
    d = np.load(path)
    for op in OPS:
        got = ctx.image_morph(int(d["width"]), int(d["height"]), d["offs"], d["events"], float(d["radius"]), op)
        assert np.array_equal(got[0], d[f"{op}_offs"]) and np.array_equal(got[1], d[f"{op}_events"]), op


@pytest.mark.gpu
@pytest.mark.parametrize("seed", range(4))
def test_gpu_image_matches_oracle(ctx, oracle, seed):
    rng = np.random.default_rng(100 + seed)
    for trial in range(12):
        w, h = int(rng.integers(1, 700)), int(rng.integers(1, 300))
        r = float(rng.choice([0.0, 1.0, 2.5, 4.0, 9.75, 17.0, 40.0]))
        offs, ev = blobs(w, h, int(rng.integers(0, 60)), int(rng.integers(1, 1 << 30)), rmax=30,
                         noise=float(rng.choice([0.0, 0.02])))
        for op in OPS:
            got = ctx.image_morph(w, h, offs, ev, r, op)
            want = oracle.image_morph(w, h, offs, ev, r, OPS[op])
            assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1]), (w, h, r, op)


@pytest.mark.gpu
def test_gpu_image_edge_shapes(ctx, oracle):
    cases = [np.zeros((5, 7), bool), np.ones((5, 7), bool), np.ones((1, 1), bool), np.zeros((1, 9), bool)]
    m = np.zeros((30, 40), bool)
    m[:, 0] = m[:, -1] = m[0, :] = True  # pixels on the image border
    cases.append(m)
    cases.append(np.ones((40, 3), bool))
    for mask in cases:
        h, w = mask.shape
        offs, ev = from_mask(mask)
        for r in (0.0, 1.0, 3.0, 50.0):
            for op in OPS:
                got = ctx.image_morph(w, h, offs, ev, r, op)
                want = oracle.image_morph(w, h, offs, ev, r, OPS[op])
                assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1]), (mask.shape, r, op)


@pytest.mark.gpu
def test_gpu_image_capacity_and_argument_checks(ctx, vo):
    offs, ev = blobs(50, 40, 10, 5)
    out_o = np.zeros(41, np.int32)
    out_e = np.zeros(2, np.int32)
    p = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))  # noqa: E731
    rc = vo.lib().vo_image_morph(ctx.handle, 0, 3.0, 50, 40, p(offs), p(ev), p(out_o), p(out_e), 2)
    assert rc == vo.VO_ERANGE and out_o[-1] > 2  # the required count is reported
    want = ctx.image_morph(50, 40, offs, ev, 3.0, "dilation")
    assert out_o[-1] == want[0][-1]
    bad = ev.copy()
    bad[1] = bad[0]  # events must increase strictly
    rc = vo.lib().vo_image_morph(ctx.handle, 0, 3.0, 50, 40, p(offs), p(bad), p(out_o), p(out_e), 2)
    assert rc == vo.VO_EINVAL
    rc = vo.lib().vo_image_morph(ctx.handle, 0, 3.0 - 1e-15, 50, 40, p(offs), p(ev), p(out_o), p(out_e), 2)
    assert rc == vo.VO_ERADIUS
    rc = vo.lib().vo_image_morph(ctx.handle, 9, 3.0, 50, 40, p(offs), p(ev), p(out_o), p(out_e), 2)
    assert rc == vo.VO_EINVAL


@pytest.mark.parametrize("path", GOLDEN2D_F64, ids=lambda p: os.path.basename(p)[:-4])
@pytest.mark.parametrize("op", list(OPS))
def test_oracle_image_f64_matches_reference_fixture(oracle, path, op):
    d = np.load(path)
    got = oracle.image_morph_f64(int(d["width"]), int(d["height"]), d["offs"], d["events"], float(d["radius"]),
                                 OPS[op])
    assert np.array_equal(got[0], d[f"{op}_offs"]) and np.array_equal(got[1], d[f"{op}_events"])


def test_oracle_image_f64_matches_reference_build(oracle):
    if not oracle.ref2d_available():
        pytest.skip("reference sources absent: pinned by the fixtures instead")
    rng = np.random.default_rng(4)
    for trial in range(40):
        w, h = int(rng.integers(1, 60)), int(rng.integers(1, 60))
        offs, ev = random_f64(w, h, int(rng.integers(1, 1 << 30)), int(rng.integers(0, 6)))
        for op, r in (("dilate", float(rng.choice([0.0, 0.02, 0.1]))), ("erode", float(rng.choice([0.0, 1.0, 3.5]))),
                      ("open", 0.05), ("close", 0.04)):
            a = oracle.image_morph_f64(w, h, offs, ev, r, op)
            b = oracle.ref_image_morph_f64(w, h, offs, ev, r, op)
            assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), (trial, w, h, r, op)


@pytest.mark.gpu
@pytest.mark.parametrize("path", GOLDEN2D_F64, ids=lambda p: os.path.basename(p)[:-4])
def test_gpu_image_f64_matches_reference_fixture(ctx, path):
    d = np.load(path)
    for op in OPS:
        got = ctx.image_morph_f64(int(d["width"]), int(d["height"]), d["offs"], d["events"], float(d["radius"]), op)
        assert np.array_equal(got[0], d[f"{op}_offs"]) and np.array_equal(got[1], d[f"{op}_events"]), op


@pytest.mark.gpu
def test_gpu_image_f64_matches_oracle(ctx, oracle):
    rng = np.random.default_rng(9)
    for trial in range(16):
        w, h = int(rng.integers(1, 400)), int(rng.integers(1, 300))
        offs, ev = random_f64(w, h, int(rng.integers(1, 1 << 30)), int(rng.integers(0, 8)))
        for op, r in (("dilation", float(rng.choice([0.0, 0.01, 0.05]))), ("erosion", float(rng.choice([0.0, 2.0, 6.5]))),
                      ("opening", 0.02), ("closing", 0.03)):
            got = ctx.image_morph_f64(w, h, offs, ev, r, op)
            want = oracle.image_morph_f64(w, h, offs, ev, r, OPS[op])
            assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1]), (trial, w, h, r, op)
    for mask_rows in ([[]] * 5, [[0.0, 7.0]] * 5, [[0.0, 0.0], [7.0, 7.0], [2.0, 5.0], [], [0.0, 7.0]]):
        offs = np.cumsum([0] + [len(r) for r in mask_rows]).astype(np.int32)
        ev = np.array([v for r in mask_rows for v in r], np.float64)
        for op in OPS:
            got = ctx.image_morph_f64(7, len(mask_rows), offs, ev, 0.3, op)
            want = oracle.image_morph_f64(7, len(mask_rows), offs, ev, 0.3, OPS[op])
            assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1]), (mask_rows, op)
