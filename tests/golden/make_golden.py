"""Regenerates the golden fixtures in tests/golden/ from the reference itself.

Runs the reference's own vor3d sources (compiled unmodified into
oracle/_ref/libvor3d_ref.so by ``make -C oracle ref``) on small seeded
inputs and stores inputs and outputs as .npz; likewise its vor2d
CompressedImage (oracle/_ref/libvor2d_ref.so) on seeded images, into
tests/golden/2d/. The reference source tree is
needed to build that library, so this script runs in the development
container only; the fixtures it writes travel with the repository and pin the
oracle restatement wherever the reference itself is absent.

Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
import voroffset_gb300 as V  # noqa: E402

# (name, synthetic spec, radius): small grids, uniform and lognormal spheres,
# cylinders, a non-integer radius and a padded dexelized torus.
CASES = [
    ("spheres48_r5", V.SynthSpec(48, n_spheres=24, s_rmin=3, s_rmax=14, seed=11), 5.0),
    ("cyl40_r6p5", V.SynthSpec(40, n_cyl=12, c_rmin=1, c_rmax=4, seed=12), 6.5),
    ("mixed56_r8", V.SynthSpec(56, n_spheres=20, sphere_dist="lognormal", s_median=6, s_sigma=0.5,
                               s_rmin=2, s_rmax=20, n_cyl=8, c_rmin=1, c_rmax=3, seed=13), 8.0),
    ("spheres32_r3p7", V.SynthSpec(32, n_spheres=10, s_rmin=2, s_rmax=10, seed=14), 3.7),
]
OPS = ["dilation", "erosion", "opening", "closing"]

# 2D images: (name, width, height, blob count, seed, pixel noise, radius)
IMAGE_CASES = [
    ("blobs64x48_r4", 64, 48, 14, 21, 0.0, 4.0),
    ("blobs97x61_r6p5", 97, 61, 20, 22, 0.0, 6.5),
    ("noisy40x33_r2p5", 40, 33, 6, 23, 0.15, 2.5),
    ("thin1x50_r3", 1, 50, 3, 24, 0.3, 3.0),
]
IMAGE_OPS = {"dilation": "dilate", "erosion": "erode", "opening": "open", "closing": "close"}
# FP64 twin (DoubleCompressedImage): (name, width, height, seed, spans per row, radius); dilation
# scales the radius by the row count, erosion does not
IMAGE64_CASES = [
    ("f64_50x40_r0p05", 50, 40, 31, 3, 0.05),
    ("f64_33x70_r1p5", 33, 70, 32, 4, 1.5),
]


def main():
    O.build(ref=True)
    for name, spec, r in CASES:
        grid, offs, z = V.synth_volume(spec)
        _write(name, grid, offs, z, r)
    # dexelized torus (the dexelization itself is the oracle restatement:
    # the reference's Dexelize.cpp needs geogram, which is absent)
    verts, tris = V.synth_torus(64, 16, 0.30, 0.10, 0.01, seed=5)
    og, offs, z = O.dexelize(verts, tris, num_dexels=40, padding=4)
    grid = V.Grid(og.nx, og.ny, og.origin, og.extent, og.spacing, og.padding)
    _write("torus40_p4_r3", grid, offs, z, 3.0, verts=verts, tris=tris)
    sys.path.insert(0, os.path.dirname(HERE))
    from imageutil import blobs
    for name, w, h, n, seed, noise, r in IMAGE_CASES:
        offs, ev = blobs(w, h, n, seed, noise=noise)
        out = {"width": w, "height": h, "radius": r, "offs": offs, "events": ev}
        for op, rop in IMAGE_OPS.items():
            out[f"{op}_offs"], out[f"{op}_events"] = O.ref_image_morph(w, h, offs, ev, r, rop)
        path = os.path.join(HERE, "2d", f"{name}.npz")
        np.savez_compressed(path, **out)
        print(path, os.path.getsize(path), "bytes")
    from imageutil import random_f64
    for name, w, h, seed, k, r in IMAGE64_CASES:
        offs, ev = random_f64(w, h, seed, k)
        out = {"width": w, "height": h, "radius": r, "offs": offs, "events": ev}
        for op, rop in IMAGE_OPS.items():
            out[f"{op}_offs"], out[f"{op}_events"] = O.ref_image_morph_f64(w, h, offs, ev, r, rop)
        path = os.path.join(HERE, "2d", f"{name}.npz")
        np.savez_compressed(path, **out)
        print(path, os.path.getsize(path), "bytes")


def _write(name, grid, offs, z, r, **extra):
    og = O.Grid(grid.nx, grid.ny, grid.origin, grid.extent, grid.spacing, grid.padding)
    out = {"nx": grid.nx, "ny": grid.ny, "origin": np.array(grid.origin), "extent": np.array(grid.extent),
           "spacing": grid.spacing, "padding": grid.padding, "radius": r, "offs": offs, "z": z}
    for op in OPS:
        o, zz, *_ = O.ref_morph(og, offs, z, r, op, "ours", threads=1)
        out[f"{op}_offs"], out[f"{op}_z"] = o, zz
    o, zz, *_ = O.ref_morph(og, offs, z, r, "dilation", "brute_force", threads=1)
    out["brute_offs"], out["brute_z"] = o, zz
    out.update(extra)
    path = os.path.join(HERE, f"{name}.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
