"""Known-answer tests of the ray-casting rules of create_dexels / compute_sign
(Dexelize.cpp:56-92 SOS orientation and point_in_triangle_2d, 107-121
orient_2d_inexact, 166-225 hits sorted and divided by the spacing), on meshes
whose geometry makes every dexel ray pass exactly through shared edges or
shared vertices of a triangulated sheet:

* every interior ray crosses each sheet exactly once (the simulation-of-
  simplicity tie rule gives a shared edge or vertex to exactly one triangle);
* triangles whose projection onto the grid has zero area never count;
* a ray that meets the mesh an odd number of times keeps its pairs only, and
  the column is counted as odd (vo_dexelize_odd_columns).

The oracle is checked against these answers on the CPU; the GPU rasteriser
against the same answers and the oracle, bit for bit."""
from __future__ import annotations

import numpy as np
import pytest


def sheet(xs, ys, z, flip=False, seed=0):
    """Triangulated grid of vertices xs x ys at height z; each cell's diagonal
    direction is drawn from `seed`."""
    rng = np.random.default_rng(seed)
    nxv, nyv = len(xs), len(ys)
    verts = np.array([(x, y, z) for y in ys for x in xs], dtype=np.float64)
    tris = []
    for j in range(nyv - 1):
        for i in range(nxv - 1):
            a, b, c, d = i + nxv * j, i + 1 + nxv * j, i + 1 + nxv * (j + 1), i + nxv * (j + 1)
            t = [(a, b, c), (a, c, d)] if rng.integers(0, 2) else [(a, b, d), (b, c, d)]
            tris += [(p, r, q) if flip else (p, q, r) for p, q, r in t]
    return verts, np.array(tris, dtype=np.int32)


def merge(*parts):
    verts, tris, off = [], [], 0
    for v, t in parts:
        verts.append(v)
        tris.append(t + off)
        off += len(v)
    return np.concatenate(verts), np.concatenate(tris)


def bbox_anchor(x, y, z):
    """An unused vertex that fixes the bounding box's lower corner (and so the grid origin)."""
    return np.array([[x, y, z]], dtype=np.float64), np.zeros((0, 3), dtype=np.int32)


def two_sheets(xs, ys, seed):
    return merge(sheet(xs, ys, 1.0, flip=True, seed=seed), sheet(xs, ys, 3.0, seed=seed + 1))


# name -> (mesh, spacing, expected full columns [1, 3] as a set of (x, y), columns that may hold either
# nothing or [1, 3] (rays on the sheets' outer boundary, decided by the tie rule))
def cases():
    out = {}
    # rays through every cell's diagonal (edge ties): vertices on integers, centres at cell centres
    xs = np.arange(0.0, 5.0)
    v, t = two_sheets(xs, xs, seed=3)
    out["diagonal edges"] = ((v, t), 1.0, {(i, j) for i in range(4) for j in range(4)}, set())
    # rays through vertices: vertices at the dexel centres (i + 0.5, j + 0.5)
    hs = np.arange(0.5, 5.0)
    v, t = merge(two_sheets(hs, hs, seed=5), bbox_anchor(0.0, 0.0, 1.0))
    interior = {(i, j) for i in range(1, 4) for j in range(1, 4)}
    boundary = {(i, j) for i in range(5) for j in range(5)} - interior
    out["shared vertices"] = ((v, t), 1.0, interior, boundary)
    # rays through the midpoints of axis-aligned edges: vertex rows on centre rows, columns on integers
    v, t = merge(two_sheets(np.arange(0.0, 5.0), hs, seed=7), bbox_anchor(0.0, 0.0, 1.0))
    interior = {(i, j) for i in range(4) for j in range(1, 4)}
    boundary = {(i, j) for i in range(4) for j in (0, 4)}
    out["axis-aligned edges"] = ((v, t), 1.0, interior, boundary)
    # the same with vertical (zero projected area) triangles standing on the ray lines: they never count
    walls = []
    for j in range(1, 4):
        y = j + 0.5
        walls.append((np.array([(0.0, y, 1.0), (4.0, y, 1.0), (2.0, y, 3.0)]), np.array([[0, 1, 2]], np.int32)))
    v2, t2 = merge((v, t), *walls)
    out["axis-aligned edges with vertical walls"] = ((v2, t2), 1.0, interior, boundary)
    # spacing 0.5: the rays of the diagonal-edge case plus rays through vertices and axis-aligned edges
    v, t = two_sheets(np.arange(0.0, 5.0), np.arange(0.0, 5.0), seed=9)
    full = {(i, j) for i in range(8) for j in range(8)}
    out["half spacing"] = ((v, t), 0.5, full, set())
    return out


CASES = cases()


def check_answer(g, offs, z, spacing, full, either):
    assert g.spacing == spacing
    for j in range(g.ny):
        for i in range(g.nx):
            c = i + g.nx * j
            vals = z[2 * offs[c]:2 * offs[c + 1]]
            if (i, j) in full:
                assert vals.tolist() == [1.0 / spacing, 3.0 / spacing], f"column {(i, j)}: {vals}"
            elif (i, j) in either:
                assert vals.tolist() in ([], [1.0 / spacing, 3.0 / spacing]), f"column {(i, j)}: {vals}"
            else:
                assert vals.size == 0, f"column {(i, j)}: {vals}"


@pytest.mark.parametrize("name", list(CASES))
def test_oracle_dexelization_known_answers(oracle, name):
    (verts, tris), sp, full, either = CASES[name]
    g, offs, z = oracle.dexelize(verts, tris, num_dexels=-1, padding=0, spacing=sp)
    check_answer(g, offs, z, sp, full, either)


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(CASES))
def test_gpu_dexelization_known_answers(ctx, oracle, name):
    (verts, tris), sp, full, either = CASES[name]
    v = ctx.dexelize(verts, tris, num_dexels=-1, padding=0, spacing=sp)
    offs, z = ctx.download(v)
    og, wo, wz = oracle.dexelize(verts, tris, num_dexels=-1, padding=0, spacing=sp)
    assert np.array_equal(offs, wo) and np.array_equal(z, wz)
    check_answer(og, offs, z, sp, full, either)
    assert ctx.dexelize_odd_columns() == 0
    v.free()


def test_oracle_open_sheet_keeps_pairs_only(oracle):
    verts, tris = sheet(np.arange(0.0, 5.0), np.arange(0.0, 5.0), 2.0, seed=1)
    v2, t2 = merge((verts, tris), bbox_anchor(0.0, 0.0, 0.0))
    g, offs, z = oracle.dexelize(v2, t2, num_dexels=-1, padding=1, spacing=1.0)
    assert offs[-1] == 0  # one hit per ray: nothing pairs up


@pytest.mark.gpu
def test_gpu_open_sheet_counts_odd_columns(ctx, oracle):
    # an open mesh: one sheet at z = 2 over 4 x 4 columns and a second one at z = 4 over a 2 x 2 corner
    # of them; 12 rays meet it once (odd: the hit is dropped), the corner's 4 rays twice ([2, 4])
    a = sheet(np.arange(0.0, 5.0), np.arange(0.0, 5.0), 2.0, seed=1)
    b = sheet(np.arange(0.0, 3.0), np.arange(0.0, 3.0), 4.0, seed=2)
    verts, tris = merge(a, b, bbox_anchor(0.0, 0.0, 0.0))
    v = ctx.dexelize(verts, tris, num_dexels=-1, padding=1, spacing=1.0)
    offs, z = ctx.download(v)
    og, wo, wz = oracle.dexelize(verts, tris, num_dexels=-1, padding=1, spacing=1.0)
    assert np.array_equal(offs, wo) and np.array_equal(z, wz)
    assert ctx.dexelize_odd_columns() == 12  # the 2 x 2 corner has two hits: [2, 4]
    assert offs[-1] == 4 and np.all(z.reshape(-1, 2) == [2.0, 4.0])
    v.free()
