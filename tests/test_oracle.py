"""The oracle restatement, pinned (CPU only).

* against the golden fixtures written by the reference itself
  (tests/golden/make_golden.py), everywhere;
* against the reference compiled unmodified (oracle/_ref), where the
  reference sources exist;
* plus the properties the reference's own cross-checks give: the two methods
  agree (`ours` vs `brute_force`, offset3d.cpp:47,105-112), a dilation
  contains its input, an erosion is inside it, opening is inside the input
  and closing around it, a larger radius dilates further, radius 0 is the
  identity union.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN, assert_same, load_golden, ogrid

OPS = ["dilation", "erosion", "opening", "closing"]


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: p.split("/")[-1][:-4])
@pytest.mark.parametrize("op", OPS)
def test_oracle_matches_golden(oracle, path, op):
    grid, d = load_golden(path)
    g = ogrid(oracle, grid)
    got = oracle.morph(g, d["offs"], d["z"], float(d["radius"]), op)
    assert_same(got, (d[f"{op}_offs"], d[f"{op}_z"]), tol=1e-9, what=f"{path}:{op}")


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: p.split("/")[-1][:-4])
def test_oracle_brute_matches_golden(oracle, path):
    grid, d = load_golden(path)
    g = ogrid(oracle, grid)
    got = oracle.morph(g, d["offs"], d["z"], float(d["radius"]), "dilation", "brute")
    # brute force and the separable scheme differ only in FP64 rounding
    assert_same(got, (d["brute_offs"], d["brute_z"]), tol=1e-9, what=f"{path}:brute")


def test_golden_torus_dexelization_is_reproduced(oracle, vo):
    import os
    from conftest import ROOT
    d = np.load(os.path.join(ROOT, "tests", "golden", "torus40_p4_r3.npz"))
    g, offs, z = oracle.dexelize(d["verts"], d["tris"], num_dexels=40, padding=4)
    assert (g.nx, g.ny) == (int(d["nx"]), int(d["ny"]))
    assert np.array_equal(offs, d["offs"]) and np.array_equal(z, d["z"])


REF_CASES = [
    (dict(n=64, n_spheres=30, s_rmin=4, s_rmax=20, seed=101), 6.0),
    (dict(n=72, n_cyl=40, c_rmin=1, c_rmax=4, seed=102), 9.25),
    (dict(n=80, n_spheres=60, sphere_dist="lognormal", s_median=8, s_sigma=0.5, s_rmin=2, s_rmax=30,
          n_cyl=20, seed=103), 12.0),
]


@pytest.mark.parametrize("case", range(len(REF_CASES)))
@pytest.mark.parametrize("op", OPS)
def test_oracle_matches_reference_build(oracle, vo, case, op):
    if not oracle.ref_available():
        pytest.skip("reference sources absent: pinned by the golden fixtures instead")
    spec, r = REF_CASES[case]
    grid, offs, z = vo.synth_volume(vo.SynthSpec(**spec))
    g = ogrid(oracle, grid)
    got = oracle.morph(g, offs, z, r, op)
    ref = oracle.ref_morph(g, offs, z, r, op, "ours", threads=4)
    assert_same(got, ref[:2], tol=1e-9, what=f"{spec}:{op}")


def test_methods_agree(oracle, vo):
    grid, offs, z = vo.synth_volume(vo.SynthSpec(60, n_spheres=25, s_rmin=3, s_rmax=18, seed=7))
    g = ogrid(oracle, grid)
    a = oracle.morph(g, offs, z, 7.5, "dilation", "separable")
    b = oracle.morph(g, offs, z, 7.5, "dilation", "brute")
    assert_same(a, b, tol=1e-9)


def _covered(offs, z, c, lo, hi):
    s = z[2 * offs[c]:2 * offs[c + 1]].reshape(-1, 2)
    return bool(np.any((s[:, 0] <= lo) & (hi <= s[:, 1])))


def test_dilation_contains_input_erosion_inside(oracle, vo):
    grid, offs, z = vo.synth_volume(vo.SynthSpec(48, n_spheres=20, s_rmin=3, s_rmax=12, seed=9))
    g = ogrid(oracle, grid)
    do, dz = oracle.morph(g, offs, z, 4.0, "dilation")
    eo, ez = oracle.morph(g, offs, z, 4.0, "erosion")
    for c in range(grid.ncols):
        for a, b in z[2 * offs[c]:2 * offs[c + 1]].reshape(-1, 2):
            assert _covered(do, dz, c, a, b)
        for a, b in ez[2 * eo[c]:2 * eo[c + 1]].reshape(-1, 2):
            assert _covered(offs, z, c, a, b)


def _covered_eps(offs, z, c, lo, hi, eps):
    s = z[2 * offs[c]:2 * offs[c + 1]].reshape(-1, 2)
    return bool(np.any((s[:, 0] - eps <= lo) & (hi <= s[:, 1] + eps)))


def _inside(ao, az, bo, bz, eps=0.0):
    """Every interval of volume A lies in one interval of volume B (same grid),
    up to eps at either end."""
    for c in range(len(ao) - 1):
        s = bz[2 * bo[c]:2 * bo[c + 1]].reshape(-1, 2)
        for a, b in az[2 * ao[c]:2 * ao[c + 1]].reshape(-1, 2):
            if not np.any((s[:, 0] - eps <= a) & (b <= s[:, 1] + eps)):
                return False
    return True


@pytest.mark.parametrize("r", [2.5, 6.0])
def test_opening_inside_input_inside_closing(oracle, vo, r):
    """Opening is anti-extensive and closing extensive (the structuring element
    holds its centre), as the reference's chains of offset3d.cpp:124-133 give,
    up to the rounding of an endpoint moved down by H and up again (a few ulps:
    at most 5.3e-15 here). Closing is extensive only away from the volume's
    border: its erosion takes everything outside the grid and outside the z
    range as empty (Voronoi.cpp:8-89), so within r of them it erodes material
    the dilation could not restore."""
    grid, offs, z = vo.synth_volume(vo.SynthSpec(40, ny=36, n_spheres=18, s_rmin=2, s_rmax=10, n_cyl=3, seed=21))
    g = ogrid(oracle, grid)
    oo, oz = oracle.morph(g, offs, z, r, "opening")
    co, cz = oracle.morph(g, offs, z, r, "closing")
    assert _inside(oo, oz, offs, z, eps=1e-12)
    m = int(np.ceil(r)) + 1
    zmax = grid.extent[2]
    checked = 0
    for c in range(grid.ncols):
        x, y = c % grid.nx, c // grid.nx
        if not (m <= x < grid.nx - m and m <= y < grid.ny - m):
            continue
        for a, b in z[2 * offs[c]:2 * offs[c + 1]].reshape(-1, 2):
            if a > r + 1 and b < zmax - r - 1:
                assert _covered_eps(co, cz, c, a, b, 1e-12), (c, a, b)
                checked += 1
    assert checked > 50


def test_dilation_grows_with_radius(oracle, vo):
    """A larger ball holds the smaller one, so its dilation holds the other's."""
    grid, offs, z = vo.synth_volume(vo.SynthSpec(40, ny=32, n_spheres=15, s_rmin=2, s_rmax=9, n_cyl=2, seed=22))
    g = ogrid(oracle, grid)
    prev = None
    for r in (1.0, 2.5, 4.0, 7.25):
        cur = oracle.morph(g, offs, z, r, "dilation")
        if prev is not None:
            assert _inside(prev[0], prev[1], cur[0], cur[1]), r
        prev = cur


def test_radius_zero_is_identity(oracle, vo):
    grid, offs, z = vo.synth_volume(vo.SynthSpec(32, n_spheres=10, s_rmin=2, s_rmax=9, seed=4))
    g = ogrid(oracle, grid)
    assert_same(oracle.morph(g, offs, z, 0.0, "dilation"), (offs, z))


def test_empty_volume(oracle):
    g = oracle.Grid(8, 5, (0, 0, 0), (8, 5, 10), 1.0, 0)
    offs = np.zeros(41, np.int32)
    o, zz = oracle.morph(g, offs, np.zeros(0), 3.0, "dilation")
    assert o[-1] == 0
    # erosion of nothing is nothing; the complement border keeps it empty
    o, zz = oracle.morph(g, offs, np.zeros(0), 3.0, "erosion")
    assert o[-1] == 0


@pytest.mark.parametrize("op", OPS)
@pytest.mark.parametrize("padded", [False, True])
def test_morph_columns_equals_whole_volume(oracle, vo, op, padded):
    """The selected-columns oracle (used to check full-size GPU results on a
    sample) returns exactly the whole-volume result's columns, for every op,
    at the grid edges too; on an unpadded grid the closing's complement leaves
    [zmin, zmax] and produces inverted pairs, which it normalises the same way."""
    g, offs, z = vo.synth_volume(vo.SynthSpec(56, ny=44, n_spheres=30, s_rmin=2, s_rmax=12, n_cyl=6, seed=61))
    grid = ogrid(oracle, g)
    if padded:
        grid = oracle.Grid(g.nx, g.ny, (0.0, 0.0, -6.0), g.extent, 1.0, 3)
    r = 5.5
    want = oracle.morph(grid, offs, z, r, op)
    rng = np.random.default_rng(5)
    cols = np.unique(np.concatenate([rng.integers(0, g.ncols, 40), [0, g.nx - 1, g.ncols - 1]])).astype(np.int32)
    so, sz = oracle.morph_columns(grid, offs, z, r, op, cols)
    wo, wz = want
    for i, c in enumerate(cols):
        assert np.array_equal(sz[2 * so[i]:2 * so[i + 1]], wz[2 * wo[c]:2 * wo[c + 1]]), f"{op} column {c}"
