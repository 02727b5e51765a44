"""Seeded 2D test images in the row-span form of the reference's CompressedImage:
`height` rows of `width` pixels, each row a sorted list of half-open pixel
spans given as events [a0, b0, a1, b1, ...], in CSR form (row_offs counts
events)."""
from __future__ import annotations

import numpy as np


def from_mask(mask):
    """CSR events of a boolean mask [height, width]."""
    h, w = mask.shape
    offs = [0]
    ev = []
    for i in range(h):
        row = np.concatenate([[False], mask[i], [False]]).astype(np.int8)
        ch = np.nonzero(np.diff(row))[0]
        ev.extend(ch.tolist())
        offs.append(len(ev))
    return np.array(offs, np.int32), np.array(ev, np.int32)


def to_mask(w, h, offs, ev):
    m = np.zeros((h, w), bool)
    for i in range(h):
        e = ev[offs[i]:offs[i + 1]]
        for a, b in zip(e[0::2], e[1::2]):
            m[i, a:b] = True
    return m


def blobs(w, h, n, seed, rmax=12.0, noise=0.0):
    """Union of seeded discs and axis-aligned rectangles, optionally with pixel noise."""
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w]
    m = np.zeros((h, w), bool)
    for _ in range(n):
        cy, cx = rng.uniform(-0.1 * h, 1.1 * h), rng.uniform(-0.1 * w, 1.1 * w)
        if rng.random() < 0.6:
            r = rng.uniform(1.0, rmax)
            m |= (yy - cy) ** 2 + (xx - cx) ** 2 <= r * r
        else:
            hy, hx = rng.uniform(0.5, rmax), rng.uniform(0.5, rmax)
            m |= (np.abs(yy - cy) <= hy) & (np.abs(xx - cx) <= hx)
    if noise > 0:
        m ^= rng.random((h, w)) < noise
    return from_mask(m)


def random_f64(w, h, seed, max_spans=4):
    """Rows of sorted FP64 events in [0, w] (closed spans, some zero-length and touching)."""
    rng = np.random.default_rng(seed)
    offs = [0]
    ev = []
    for _ in range(h):
        k = int(rng.integers(0, max_spans + 1))
        v = np.sort(rng.uniform(0, w, 2 * k))
        if k and rng.random() < 0.2:
            v[1] = v[0]  # a point span
        if k > 1 and rng.random() < 0.2:
            v[2] = v[1]  # touching spans
        ev.extend(v.tolist())
        offs.append(len(ev))
    return np.array(offs, np.int32), np.array(ev, np.float64)
