"""The C++ host layer on the GPU: VoronoiMorphoGpu called through the
reference's VoronoiMorpho interface (Voronoi.h:13-44), and the offset3d_gpu CLI
(app/cli3d/offset3d.cpp:104-136) run on the torus configuration from an OBJ
file, both compared with the oracle bit for bit."""
from __future__ import annotations

import json
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, assert_same, ogrid
from hostutil import build_host_check, read_csr_volume, read_obj, read_text_volume, write_text_volume

pytestmark = pytest.mark.gpu

CLI = os.path.join(ROOT, "voroffset_gb300", "bin", "offset3d_gpu")


@pytest.fixture(scope="module")
def host_check(tmp_path_factory, vo):
    return build_host_check(str(tmp_path_factory.mktemp("host")))


@pytest.mark.parametrize("op,method", [("erosion", "fast"), ("erosion", "separable"), ("dilation", "fast"),
                                       ("closing", "fast"), ("opening", "separable")])
def test_voronoi_morpho_gpu_directly(host_check, vo, oracle, tmp_path, op, method):
    grid, offs, z = vo.synth_volume(vo.SynthSpec(48, ny=40, n_spheres=25, s_rmin=2, s_rmax=10, n_cyl=4, seed=21))
    src, dst = tmp_path / "in.txt", tmp_path / "out.txt"
    write_text_volume(src, grid, offs, z)
    subprocess.run([host_check, "morph", op, method, "4.5", str(src), str(dst)], check=True)
    head, o, zz = read_text_volume(dst)
    assert head[:2] == (48, 40)
    assert_same((o, zz), oracle.morph(ogrid(oracle, grid), offs, z, 4.5, op), tol=0.0, what=f"{op} {method}")


def write_obj(path, verts, tris):
    with open(path, "w") as fh:
        for v in verts:
            fh.write("v %.17g %.17g %.17g\n" % tuple(v))
        for t in tris:
            fh.write("f %d %d %d\n" % (t[0] + 1, t[1] + 1, t[2] + 1))


@pytest.mark.parametrize("op", ["dilation", "closing"])
def test_offset3d_cli_on_the_torus_configuration(vo, oracle, tmp_path, op):
    """-n 256 -p 10 -r 8 on the 256 x 64-quad torus with seeded normal noise."""
    verts, tris = vo.synth_torus(256, 64, 0.30, 0.10, 0.01, seed=1)
    mesh = tmp_path / "torus.obj"
    write_obj(mesh, verts, tris)
    out_vol, out_mesh, out_json = tmp_path / "out.csr", tmp_path / "out.obj", tmp_path / "out.json"
    subprocess.run([CLI, str(mesh), "-n", "256", "-p", "10", "-r", "8", "-x", op, "-o", str(out_mesh), "-j",
                    str(out_json), "-s", str(out_vol)], check=True)
    og, offs, z = oracle.dexelize(verts, tris, num_dexels=256, padding=10)
    want = oracle.morph(og, offs, z, 8.0, op)
    head, o, zz = read_csr_volume(out_vol)
    assert head[:2] == (og.nx, og.ny) and head[5] == 10
    assert_same((o, zz), want, tol=0.0, what=f"offset3d_gpu {op}")
    info = json.load(open(out_json))
    assert info["operation"] == op and info["grid_size"] == [og.nx, og.ny]
    assert info["num_segments"] == int(offs[-1]) and info["output_segments"] == int(o[-1])
    verts_out, faces = read_obj(out_mesh)
    assert len(faces) >= 2 * int(o[-1])  # at least the top and bottom of every output segment
