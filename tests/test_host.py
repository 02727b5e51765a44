"""The C++ host layer without a GPU (voroffset_gb300/host, linked into
libvoroffset_gpu.so): CompressedVolume's text format (CompressedVolume.cpp:116-152)
and binary CSR dump round-trip, numSegments / get_volume
(CompressedVolume.cpp:61-83), and the mesh writers (dexel_dump,
Dexelize.cpp:312-351) checked by face and vertex counts on known volumes."""
from __future__ import annotations

import subprocess

import numpy as np
import pytest

from hostutil import build_host_check, read_csr_volume, read_obj, read_text_volume, write_text_volume


@pytest.fixture(scope="module")
def host_check(tmp_path_factory, vo):
    return build_host_check(str(tmp_path_factory.mktemp("host")))


def vol(vo, nx, ny, cols, zmax=8.0):
    offs = np.zeros(nx * ny + 1, dtype=np.int32)
    z = []
    for c in range(nx * ny):
        segs = cols.get(c, [])
        offs[c + 1] = offs[c] + len(segs)
        for a, b in segs:
            z += [a, b]
    return vo.Grid(nx, ny, (0.0, 0.0, 0.0), (float(nx), float(ny), zmax), 1.0, 0), offs, np.array(z, dtype=np.float64)


def test_text_format_round_trip(host_check, vo, tmp_path):
    grid, offs, z = vo.synth_volume(vo.SynthSpec(24, ny=17, n_spheres=12, s_rmin=2, s_rmax=8, seed=3))
    z = np.round(z * 4) / 4  # values the format's default 6 digits print exactly
    src, dst = tmp_path / "a.txt", tmp_path / "b.txt"
    write_text_volume(src, grid, offs, z, fmt="%.6g")
    subprocess.run([host_check, "roundtrip", str(src), str(dst)], check=True)
    assert open(src).read() == open(dst).read()


def test_binary_csr_round_trip_is_exact(host_check, vo, tmp_path):
    grid, offs, z = vo.synth_volume(vo.SynthSpec(40, ny=33, n_spheres=30, s_rmin=2, s_rmax=12, n_cyl=5, seed=8))
    src, csr, back = tmp_path / "a.txt", tmp_path / "a.csr", tmp_path / "b.txt"
    write_text_volume(src, grid, offs, z)
    subprocess.run([host_check, "csr", str(src), str(csr), str(back)], check=True)
    head, o2, z2 = read_csr_volume(csr)
    assert head[:2] == (40, 33) and np.array_equal(o2, offs) and np.array_equal(z2, z)
    _, o3, z3 = read_text_volume(back)
    assert np.array_equal(o3, offs) and np.array_equal(z3, z)


def test_num_segments_and_volume(host_check, vo, tmp_path):
    grid, offs, z = vo.synth_volume(vo.SynthSpec(30, n_spheres=15, s_rmin=2, s_rmax=9, seed=12))
    src = tmp_path / "a.txt"
    write_text_volume(src, grid, offs, z)
    out = subprocess.run([host_check, "stats", str(src)], check=True, capture_output=True, text=True).stdout.split()
    assert int(out[0]) == int(offs[-1])
    assert float(out[1]) == pytest.approx(float(np.sum(z[1::2] - z[0::2])), rel=1e-12)


# (columns -> segments, expected boundary faces, expected merged vertices)
SURFACES = [
    ("one box", 1, 1, {0: [(0, 2)]}, 6, 8),
    ("two equal boxes side by side", 2, 1, {0: [(0, 2)], 1: [(0, 2)]}, 10, 12),
    ("two staggered boxes", 2, 1, {0: [(0, 2)], 1: [(1, 3)]}, 12, 16),
    ("2 x 2 block", 2, 2, {0: [(0, 1)], 1: [(0, 1)], 2: [(0, 1)], 3: [(0, 1)]}, 16, 18),
    ("touching segments in one column", 1, 1, {0: [(0, 1), (1, 2)]}, 10, 12),
    ("two segments with a gap", 1, 1, {0: [(0, 1), (2, 3)]}, 12, 16),
]


@pytest.mark.parametrize("case", SURFACES, ids=[s[0] for s in SURFACES])
def test_surface_writer_face_counts(host_check, vo, tmp_path, case):
    _, nx, ny, cols, nfaces, nverts = case
    grid, offs, z = vol(vo, nx, ny, cols)
    src, obj = tmp_path / "v.txt", tmp_path / "v.obj"
    write_text_volume(src, grid, offs, z)
    subprocess.run([host_check, "surface", str(src), str(obj)], check=True)
    verts, faces = read_obj(obj)
    assert (len(faces), len(verts)) == (nfaces, nverts)
    assert len(set(verts)) == len(verts)  # merged: no two vertices at one position
    assert all(len(f) == 4 and max(f) <= len(verts) for f in faces)
    # every face edge is shared by an even number of faces when no T-junction occurs
    if case[0] != "two staggered boxes":
        edges = {}
        for f in faces:
            for k in range(4):
                e = tuple(sorted((f[k], f[(k + 1) % 4])))
                edges[e] = edges.get(e, 0) + 1
        assert all(n % 2 == 0 for n in edges.values())


def test_box_writer_and_points(host_check, vo, tmp_path):
    grid, offs, z = vol(vo, 3, 2, {0: [(0, 2)], 4: [(1, 3), (4, 5)]})
    src, obj = tmp_path / "v.txt", tmp_path / "b.obj"
    write_text_volume(src, grid, offs, z)
    subprocess.run([host_check, "boxes", str(src), str(obj)], check=True)
    verts, faces = read_obj(obj)
    assert (len(faces), len(verts)) == (6 * 3, 8 * 3)
