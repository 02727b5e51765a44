"""Trains the learned tile sizer on volumes the method itself generates.

    python -m voroffset_gb300.train_sizer [--volumes 2000] [--steps 3000] [--out voroffset_gb300/sizer_weights.f32]

Every training volume is a seeded synthetic union of spheres (uniform or
lognormal radii) and cylinders on a 64..256 square grid with a z-range up to
4096 dexels (object densities per dexel^3 over two decades); half of them are
replaced by their complement with a one-column border (the input the erosion
chain dilates), and every third one also contributes the complement of its
dilation (the input of a closing's second dilation). Each is dilated by the FP32-guarded GPU method at a radius in
[2, 64] (multiples of 0.25), and the per-tile features of the input and the
targets from the result (vo_sizer_tile_features / vo_sizer_tile_targets)
form one sample per 32 x 32 tile. Training is full-batch Adam on the device
(vo_sizer_train). The weights are written as raw little-endian float32 with a
JSON sidecar describing the run.
"""
from __future__ import annotations

import argparse
import json
import os
import time

import numpy as np

from . import Context, Grid, SynthSpec, synth_volume

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "sizer_weights.f32")


def complement(grid: Grid, offs: np.ndarray, z: np.ndarray):
    """Complement of every column on [zmin, zmax] with a border of full columns
    (the shape of the erosion chain's dilation input, Voronoi.cpp:38-70,
    negate_ray of MorphologyOperators.cpp:230-259, without its rare drop of a
    value equal to zmin or zmax)."""
    zmin = grid.origin[2] / grid.spacing - 1
    zmax = grid.origin[2] / grid.spacing + 2 * grid.padding + grid.extent[2] / grid.spacing + 1
    nx, ny = grid.nx, grid.ny
    idx = np.empty(2 * (nx * ny), np.int64)
    idx[0::2] = 2 * offs[:-1]
    idx[1::2] = 2 * offs[1:]
    vals = np.empty(2 * (nx * ny))
    vals[0::2] = zmin
    vals[1::2] = zmax
    zc = np.insert(z, idx, vals)
    cnt = np.diff(offs) + 1
    pairs = zc.reshape(-1, 2)
    col = np.repeat(np.arange(nx * ny), cnt)
    # An inverted pair [a, b], a > b, is left where a column's values exceed
    # [zmin, zmax]; like the method (and the reference's pass 2, which sees its
    # two endpoints), rewrite it as the points [b, b] and [a, a], then sort and
    # merge that column as closed intervals. Empty pairs of other columns are
    # kept as they are.
    inv = pairs[:, 0] > pairs[:, 1]
    if inv.any():
        bad = np.unique(col[inv])
        starts = np.concatenate([[0], np.cumsum(cnt)])
        fixed_pairs, fixed_cols = [], []
        for c in bad:
            seg = pairs[starts[c]:starts[c + 1]]
            pts = []
            for a, b in seg:
                pts += [(b, b), (a, a)] if a > b else [(a, b)]
            pts.sort()
            merged = []
            for a, b in pts:
                if merged and not (merged[-1][1] < a):
                    merged[-1][1] = max(merged[-1][1], b)
                else:
                    merged.append([a, b])
            fixed_pairs += merged
            fixed_cols += [c] * len(merged)
        drop = np.isin(col, bad)
        pairs = np.concatenate([pairs[~drop], np.array(fixed_pairs).reshape(-1, 2)])
        col = np.concatenate([col[~drop], np.array(fixed_cols, dtype=col.dtype)])
        order = np.argsort(col, kind="stable")
        pairs, col = pairs[order], col[order]
    cnt = np.bincount(col, minlength=nx * ny).reshape(ny, nx)
    # bordered grid (nx+2) x (ny+2): interior (x+1, y+1) <- (x, y); border columns full
    full = np.zeros((ny + 2, nx + 2), np.int64) + 1
    full[1:-1, 1:-1] = cnt
    offs2 = np.zeros((nx + 2) * (ny + 2) + 1, np.int32)
    offs2[1:] = np.cumsum(full.reshape(-1))
    z2 = np.empty((offs2[-1], 2))
    border = np.ones((ny + 2, nx + 2), bool)
    border[1:-1, 1:-1] = False
    bcols = np.flatnonzero(border.reshape(-1))
    z2[offs2[bcols]] = (zmin, zmax)
    icols = np.flatnonzero(~border.reshape(-1))
    starts = offs2[icols]
    rep = np.repeat(starts, cnt.reshape(-1))
    within = np.arange(len(pairs)) - np.repeat(np.cumsum(cnt.reshape(-1)) - cnt.reshape(-1), cnt.reshape(-1))
    z2[rep + within] = pairs
    g2 = Grid(nx + 2, ny + 2, grid.origin, grid.extent, grid.spacing, grid.padding)
    return g2, offs2, z2.reshape(-1)


def make_volume(rng: np.random.Generator):
    side = int(rng.choice([64, 96, 128, 192, 256]))
    zmax = float(np.exp(rng.uniform(np.log(side), np.log(4096))))  # tall columns stack many objects
    lognormal = bool(rng.integers(0, 2))
    # object densities per dexel^3, log-uniform over two decades
    vol = side * side * zmax
    ns = int(vol * np.exp(rng.uniform(np.log(5e-7), np.log(1e-4))))
    nc = int(vol * np.exp(rng.uniform(np.log(3e-8), np.log(3e-6)))) if rng.integers(0, 3) else 0
    spec = SynthSpec(side, n_spheres=max(1, ns), s_rmin=2, s_rmax=float(rng.uniform(6, 80 if lognormal else 40)),
                     n_cyl=nc, c_rmin=1, c_rmax=float(rng.uniform(1.5, 4)), seed=int(rng.integers(1, 1 << 40)),
                     sphere_dist="lognormal" if lognormal else "uniform", s_median=float(rng.uniform(4, 16)),
                     s_sigma=float(rng.uniform(0.3, 0.7)), zmax=zmax)
    g, offs, z = synth_volume(spec)
    if rng.integers(0, 2):
        g, offs, z = complement(g, offs, z)
    r = float(np.round(rng.uniform(2, 64) * 4) / 4)
    return g, offs, z, r


def generate(ctx: Context, n: int, seed: int, log_every: int = 0):
    """Features and targets of n generated volumes. Every third one also adds
    the second dilation of a closing: the complement (with border) of the
    first dilation's result, dilated by the same radius."""
    rng = np.random.default_rng(seed)
    sz = ctx.sizer(seed=1)
    feats, targs = [], []
    for i in range(n):
        g, offs, z, r = make_volume(rng)
        v = ctx.upload(g, offs, z)
        out, _ = ctx.morph(v, "dilation", r, "fast")
        feats.append(sz.features(v, r))
        targs.append(sz.targets(v, out, r))
        if i % 3 == 2:
            o1, z1 = ctx.download(out)
            g2, o2, z2 = complement(g, o1, z1)
            v2 = ctx.upload(g2, o2, z2)
            out2, _ = ctx.morph(v2, "dilation", r, "fast")
            feats.append(sz.features(v2, r))
            targs.append(sz.targets(v2, out2, r))
            out2.free()
            v2.free()
        out.free()
        v.free()
        if log_every and (i + 1) % log_every == 0:
            print(f"  {i + 1}/{n} volumes", flush=True)
    sz.free()
    return np.concatenate(feats), np.concatenate(targs)


def train(ctx: Context, feats, targs, steps: int, lr: float, seed: int = 7):
    sz = ctx.sizer(seed=seed)
    loss = sz.train(feats, targs, steps=steps, lr=lr)
    return sz, loss


def load(ctx: Context, path: str = WEIGHTS):
    """A sizer with the weights at `path` (raises if the file is missing)."""
    sz = ctx.sizer(seed=1)
    p = np.fromfile(path, dtype="<f4")
    sz.set_params(p)
    return sz


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--volumes", type=int, default=2000)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--out", default=WEIGHTS)
    a = ap.parse_args()
    with Context(0) as ctx:
        t0 = time.time()
        X, T = generate(ctx, a.volumes, a.seed, log_every=max(1, a.volumes // 10))
        t1 = time.time()
        sz, loss = train(ctx, X, T, a.steps, a.lr)
        t2 = time.time()
        pred = sz.forward(X)
        err = np.abs(pred - T).mean(0)
        sz.params().astype("<f4").tofile(a.out)
        meta = {"volumes": a.volumes, "samples": int(len(X)), "steps": a.steps, "lr": a.lr, "seed": a.seed,
                "final_loss": loss, "mean_abs_err_log2": [float(e) for e in err],
                "generate_s": round(t1 - t0, 1), "train_s": round(t2 - t1, 1)}
        with open(os.path.splitext(a.out)[0] + ".json", "w") as f:
            json.dump(meta, f, indent=1)
        print(json.dumps(meta))
        sz.free()


if __name__ == "__main__":
    main()
