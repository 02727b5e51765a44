"""CPU model of the dominance pruning of the FP32 dilation kernels.

A candidate of source column s at offset (dx, dy) is [z1 - H, z2 + H] with
H = H[|dy|][|dx|]. Its neighbour s' one lattice step toward the output column
contributes [z1' - H', z2' + H'] with H' >= H. If every segment of s lies in a
segment of s' widened by w <= H' - H, each candidate of s is inside one of s'
(in exact arithmetic on the FP64 values, hence also after rounding each
endpoint), so s can be skipped; chains of skips end at a kept candidate.
The kernels bound w from above and H' - H from below; this model does the same
with one-ulp widening and must reproduce the oracle's dilation bit for bit.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from conftest import ogrid


def _tables(R):
    Dy = int(math.floor(R))
    r = [R if d == 0 else math.sqrt(R * R - d * d) for d in range(Dy + 1)]
    Dx = [int(math.floor(v)) for v in r]
    H = {(d, a): math.sqrt(r[d] * r[d] - a * a) for d in range(Dy + 1) for a in range(Dx[d] + 1)}
    return Dy, Dx, H


def _down(v):  # a float32 value <= v
    f = np.float32(np.nextafter(v, -np.inf))
    return float(f) if float(f) <= v else float(np.nextafter(f, np.float32(-np.inf)))


def _up(v):
    f = np.float32(np.nextafter(v, np.inf))
    return float(f) if float(f) >= v else float(np.nextafter(f, np.float32(np.inf)))


def _dominance(nx, ny, cols):
    dom = np.full((4, nx * ny), -np.inf)
    for c in range(nx * ny):
        x, y = c % nx, c // nx
        if not cols[c]:
            continue
        for k, (ex, ey) in enumerate(((-1, 0), (1, 0), (0, -1), (0, 1))):
            xn, yn = x + ex, y + ey
            if not (0 <= xn < nx and 0 <= yn < ny):
                dom[k, c] = np.inf
                continue
            w = -np.inf
            for (a1, a2) in cols[c]:
                best = min([max(np.nextafter(b1 - a1, np.inf), np.nextafter(a2 - b2, np.inf))
                            for (b1, b2) in cols[xn + nx * yn]] or [np.inf])
                w = max(w, best)
            dom[k, c] = _up(w)
    return dom


def _pruned_dilation(nx, ny, cols, R):
    Dy, Dx, H = _tables(R)
    dom = _dominance(nx, ny, cols)
    dhx = {(d, a): _down(H[(d, a - 1)] - H[(d, a)]) if a >= 1 else -np.inf for (d, a) in H}
    dhy = {(d, a): _down(H[(d - 1, a)] - H[(d, a)]) if d >= 1 else -np.inf for (d, a) in H}
    out, kept, total = [], 0, 0
    for c in range(nx * ny):
        x, y = c % nx, c // nx
        cand = []
        for (d, a), h in H.items():
            for sx in ((1, -1) if a else (1,)):
                for sy in ((1, -1) if d else (1,)):
                    xs, ys = x + sx * a, y + sy * d
                    if not (0 <= xs < nx and 0 <= ys < ny):
                        continue
                    s = xs + nx * ys
                    total += len(cols[s])
                    wx = dom[0 if sx > 0 else 1, s]
                    wy = dom[2 if sy > 0 else 3, s]
                    if wx <= dhx[(d, a)] or wy <= dhy[(d, a)]:
                        continue
                    kept += len(cols[s])
                    cand += [(z1 - h, z2 + h) for (z1, z2) in cols[s]]
        cand.sort()
        u = []
        for lo, hi in cand:
            if u and lo <= u[-1][1]:
                u[-1][1] = max(u[-1][1], hi)
            else:
                u.append([lo, hi])
        out.append(u)
    return out, kept, total


@pytest.mark.parametrize("R,seed", [(1.5, 1), (3.0, 2), (4.5, 3), (6.0, 4), (5.25, 5)])
def test_pruned_union_equals_oracle(vo, oracle, R, seed):
    g, offs, z = vo.synth_volume(vo.SynthSpec(22, n_spheres=10, s_rmin=2, s_rmax=7, n_cyl=3, seed=seed))
    cols = [list(map(tuple, z[2 * offs[c]:2 * offs[c + 1]].reshape(-1, 2))) for c in range(g.ncols)]
    got, kept, total = _pruned_dilation(g.nx, g.ny, cols, R)
    wo, wz = oracle.morph(ogrid(oracle, g), offs, z, R, "dilation")
    for c in range(g.ncols):
        want = wz[2 * wo[c]:2 * wo[c + 1]].reshape(-1, 2)
        assert np.array_equal(np.array(got[c]).reshape(-1, 2), want), c
    assert kept < total  # the rule prunes something on these shapes


NLEVELS = 11


def _levels(H):
    """Dominance level thresholds of a radius, as the library's table builder
    sets them: 0, then the growths of H over one lattice step (FP32 lower
    bounds) at quantiles (l - 1/2) / (NLEVELS - 1) of their sorted list."""
    g = sorted([_down(H[(d, a - 1)] - H[(d, a)]) for (d, a) in H if a >= 1] +
               [_down(H[(d - 1, a)] - H[(d, a)]) for (d, a) in H if d >= 1])
    t = [0.0]
    for lv in range(1, NLEVELS):
        v = g[int(math.floor((lv - 0.5) / (NLEVELS - 1) * (len(g) - 1) + 0.5))] if g else 0.0
        t.append(max(v, 0.0))
    return t


def _level(dh, levels):
    """Largest level <= dh (-1: none), as the kernels quantise a pair's growth of H."""
    lv = -1
    for i, t in enumerate(levels):
        if t <= dh:
            lv = i
    return lv


def _segment_widths(nx, ny, cols):
    out = []
    for c in range(nx * ny):
        x, y = c % nx, c // nx
        ws = []
        for (a1, a2) in cols[c]:
            w4 = []
            for (ex, ey) in ((-1, 0), (1, 0), (0, -1), (0, 1)):
                xn, yn = x + ex, y + ey
                if not (0 <= xn < nx and 0 <= yn < ny):
                    w4.append(np.inf)
                    continue
                w4.append(min([max(np.nextafter(b1 - a1, np.inf), np.nextafter(a2 - b2, np.inf))
                               for (b1, b2) in cols[xn + nx * yn]] or [np.inf]))
            ws.append(w4)
        out.append(ws)
    return out


@pytest.mark.parametrize("R,seed", [(3.0, 2), (6.0, 4), (7.5, 9)])
def test_segment_masks_by_level_equal_oracle(vo, oracle, R, seed):
    """Per-segment pruning with widths compared at the quantised level of the
    pair's growth of H (the kernels' dominance masks) keeps the union exact."""
    g, offs, z = vo.synth_volume(vo.SynthSpec(20, n_spheres=12, s_rmin=2, s_rmax=7, n_cyl=3, seed=seed))
    nx, ny = g.nx, g.ny
    cols = [list(map(tuple, z[2 * offs[c]:2 * offs[c + 1]].reshape(-1, 2))) for c in range(g.ncols)]
    Dy, Dx, H = _tables(R)
    sw = _segment_widths(nx, ny, cols)
    LEVELS = _levels(H)
    lx = {(d, a): _level(_down(H[(d, a - 1)] - H[(d, a)]), LEVELS) if a >= 1 else -1 for (d, a) in H}
    ly = {(d, a): _level(_down(H[(d - 1, a)] - H[(d, a)]), LEVELS) if d >= 1 else -1 for (d, a) in H}
    kept = total = 0
    wo, wz = oracle.morph(ogrid(oracle, g), offs, z, R, "dilation")
    for c in range(nx * ny):
        x, y = c % nx, c // nx
        cand = []
        for (d, a), h in H.items():
            for sx in ((1, -1) if a else (1,)):
                for sy in ((1, -1) if d else (1,)):
                    xs, ys = x + sx * a, y + sy * d
                    if not (0 <= xs < nx and 0 <= ys < ny):
                        continue
                    s = xs + nx * ys
                    for i, (z1, z2) in enumerate(cols[s]):
                        total += 1
                        w = sw[s][i]
                        wx, wy = w[0 if sx > 0 else 1], w[2 if sy > 0 else 3]
                        if (lx[(d, a)] >= 0 and wx <= LEVELS[lx[(d, a)]]) or \
                           (ly[(d, a)] >= 0 and wy <= LEVELS[ly[(d, a)]]):
                            continue
                        kept += 1
                        cand.append((z1 - h, z2 + h))
        cand.sort()
        u = []
        for lo, hi in cand:
            if u and lo <= u[-1][1]:
                u[-1][1] = max(u[-1][1], hi)
            else:
                u.append([lo, hi])
        want = wz[2 * wo[c]:2 * wo[c + 1]].reshape(-1, 2)
        assert np.array_equal(np.array(u).reshape(-1, 2), want), c
    assert kept < total
