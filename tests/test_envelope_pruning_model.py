"""CPU model of the pass-2 pruning of the envelope form (covers_for_life in
voroffset_gb300/csrc/vo_env.cu).

Pass 2 sweeps a row of columns keeping live stadiums: pass-1 pieces (core
[a, b], label d) of the columns within reach (x - x0 <= Dx[d]); at column x a
stadium's chord is [a - H[d][x - x0], b + H[d][x - x0]] in FP64 with the
reference's tables (SeparatePower2D.cpp:295-341), and the column's output is
the union of the chords. The kernel drops a stadium once a new piece p (label
dp, entering at x) outlives it and H[dp][0] - H[d][x - x0] >= max(a_p - a,
b - b_p, 0) + a margin: the chord difference only grows along the sweep, so
p's chord holds the stadium's chord at every later column. This model sweeps
random and near-margin rows with and without the pruning (tested against every
new piece, which covers the kernel's nearest-piece candidates, and on every or
every other column) and requires identical unions, bit for bit, at every
column.
"""
from __future__ import annotations

import math

import numpy as np
import pytest


def tables(R):
    Dy = int(math.floor(R))
    r = [R if d == 0 else math.sqrt(R * R - d * d) for d in range(Dy + 1)]
    Dx = [int(math.floor(v)) for v in r]
    H = [[math.sqrt(r[d] * r[d] - t * t) for t in range(Dx[d] + 1)] for d in range(Dy + 1)]
    return Dy, Dx, H


def up(v):
    return float(np.nextafter(v, np.inf))


def down(v):
    return float(np.nextafter(v, -np.inf))


def covers_for_life(p, v, x, Dx, H, eps):
    """p = (a, b, d) entering at x; v = (a, b, d, x0): the kernel's test, with
    each rounded operation widened by one ulp in the safe direction."""
    (pa, pb, dp), (va, vb, dv, x0) = p, v
    if x + Dx[dp] < x0 + Dx[dv]:
        return False
    hv, hp = H[dv][x - x0], H[dp][0]
    m = max(up(pa - va), up(vb - pb), 0.0)
    return down(hp - hv) >= up(m + eps)


def union(chords):
    out = []
    for lo, hi in sorted(chords):
        if out and lo <= out[-1][1]:
            out[-1][1] = max(out[-1][1], hi)
        else:
            out.append([lo, hi])
    return [tuple(c) for c in out]


def sweep(cols, R, prune, period=1):
    """cols[x] = list of (a, b, d) pieces; returns the union at every column and
    the largest live state."""
    Dy, Dx, H = tables(R)
    eps = math.ldexp(max(R, 1.0), -46)
    live, outs, peak = [], [], 0
    for x, pieces in enumerate(cols):
        live = [v for v in live if x - v[3] <= Dx[v[2]]]
        if prune and x % period == 0:
            live = [v for v in live if not any(covers_for_life(p, v, x, Dx, H, eps) for p in pieces)]
        live += [(a, b, d, x) for (a, b, d) in pieces]
        peak = max(peak, len(live))
        chords = [(a - H[d][x - x0], b + H[d][x - x0]) for (a, b, d, x0) in live]
        outs.append(union(chords))
    return outs, peak


def random_row(rng, nx, R, k, scale):
    Dy = int(math.floor(R))
    cols = []
    for _ in range(nx):
        n = int(rng.integers(0, k + 1))
        cuts = np.sort(rng.uniform(0.0, scale, 2 * n))
        cols.append([(float(cuts[2 * i]), float(cuts[2 * i + 1]), int(rng.integers(0, Dy + 1))) for i in range(n)])
    return cols


@pytest.mark.parametrize("R,seed", [(3.5, 1), (6.0, 2), (9.25, 3), (16.0, 4)])
@pytest.mark.parametrize("period", [1, 2])
def test_pruned_sweep_equals_full_sweep(R, seed, period):
    rng = np.random.default_rng(seed)
    cols = random_row(rng, 70, R, 6, 60.0)
    full, peak_full = sweep(cols, R, prune=False)
    pruned, peak_pruned = sweep(cols, R, prune=True, period=period)
    assert pruned == full
    assert peak_pruned <= peak_full


def test_pruning_shrinks_the_state_of_overlapping_columns():
    """Similar columns (shifted copies of one column): newer pieces hold most
    older stadiums for life, so the live state shrinks."""
    rng = np.random.default_rng(11)
    R = 12.0
    base = random_row(rng, 1, R, 8, 80.0)[0]
    cols = [[(a + 0.01 * (x % 3), b + 0.01 * (x % 3), d) for (a, b, d) in base] for x in range(60)]
    full, peak_full = sweep(cols, R, prune=False)
    pruned, peak_pruned = sweep(cols, R, prune=True)
    assert pruned == full
    assert peak_pruned < peak_full / 2


def test_margin_cases_keep_the_union():
    """A stadium whose core overhangs a new piece by about the chord growth
    (within a few ulps either way) must never change the union when dropped."""
    R = 7.0
    Dy, Dx, H = tables(R)
    cols = []
    for x in range(40):
        pieces = []
        if x >= 1:
            g = H[0][0] - H[0][1]  # growth of a label-0 chord over one column
            for k, delta in enumerate((-3e-15, -1e-15, 0.0, 1e-15, 3e-15, 1e-9)):
                a = 10.0 * k + 0.125 * (x % 4)
                pieces.append((a, a + 1.0 + g + delta, 0))
        else:
            pieces = [(10.0 * k, 10.0 * k + 1.0, 0) for k in range(6)]
        cols.append(pieces)
    full, _ = sweep(cols, R, prune=False)
    for period in (1, 2):
        pruned, _ = sweep(cols, R, prune=True, period=period)
        assert pruned == full


@pytest.mark.parametrize("delta", [-1e-9, -1e-12, -1e-14, 1e-9, 1e-6])
def test_isolated_stadium_pruned_only_when_held(delta):
    """One stadium (column 0) and one newer piece (column 1), nothing else: the
    piece's upper end sits `delta` above what holds the stadium's chord. Below
    that (delta < 0) the stadium pokes out and must stay; with room to spare it
    is dropped, and the unions are the same either way."""
    R = 9.0
    Dy, Dx, H = tables(R)
    g = H[0][0] - H[0][1]
    cols = [[(0.0, 1.0, 0)], [(0.0, 1.0 - g + delta, 0)]] + [[] for _ in range(12)]
    full, _ = sweep(cols, R, prune=False)
    pruned, _ = sweep(cols, R, prune=True)
    assert pruned == full
    kept = sweep_live_after(cols, R, 1)
    assert (len(kept) == 2) == (delta < 1e-12)


def sweep_live_after(cols, R, x_end):
    """Live stadiums of the pruned sweep after column x_end."""
    Dy, Dx, H = tables(R)
    eps = math.ldexp(max(R, 1.0), -46)
    live = []
    for x, pieces in enumerate(cols[: x_end + 1]):
        live = [v for v in live if x - v[3] <= Dx[v[2]]]
        live = [v for v in live if not any(covers_for_life(p, v, x, Dx, H, eps) for p in pieces)]
        live += [(a, b, d, x) for (a, b, d) in pieces]
    return live
