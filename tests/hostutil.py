"""Helpers for the tests of the C++ host layer: building the check program and
reading / writing the volume file formats."""
from __future__ import annotations

import os
import struct
import subprocess

import numpy as np

from conftest import ROOT

PKG = os.path.join(ROOT, "voroffset_gb300")


def build_host_check(tmpdir: str) -> str:
    """Compiles tests/host/host_check.cpp against libvoroffset_gpu.so (its C++ host layer)."""
    exe = os.path.join(tmpdir, "host_check")
    subprocess.run(["g++", "-std=c++17", "-O1", f"-I{ROOT}/include", f"-I{PKG}/host",
                    os.path.join(ROOT, "tests", "host", "host_check.cpp"), "-o", exe, f"-L{PKG}", "-lvoroffset_gpu",
                    f"-Wl,-rpath,{PKG}", "-pthread"], check=True)
    return exe


def write_text_volume(path, grid, offs, z, fmt="%.17g"):
    """The text format of CompressedVolume::save (CompressedVolume.cpp:138-152): origin, extent,
    grid size, padding, spacing, then per column its value count and values."""
    with open(path, "w") as fh:
        fh.write(" ".join(fmt % v for v in grid.origin) + "\n")
        fh.write(" ".join(fmt % v for v in grid.extent) + "\n")
        fh.write(f"{grid.nx} {grid.ny}\n{grid.padding}\n{fmt % grid.spacing}\n")
        for c in range(grid.nx * grid.ny):
            vals = z[2 * offs[c]:2 * offs[c + 1]]
            fh.write(str(vals.size) + "".join(" " + fmt % v for v in vals) + "\n")


def read_text_volume(path):
    tok = open(path).read().split()
    origin = tuple(float(t) for t in tok[0:3])
    extent = tuple(float(t) for t in tok[3:6])
    nx, ny, pad, sp = int(tok[6]), int(tok[7]), int(tok[8]), float(tok[9])
    i = 10
    offs = [0]
    vals = []
    for _ in range(nx * ny):
        n = int(tok[i])
        vals += [float(t) for t in tok[i + 1:i + 1 + n]]
        i += 1 + n
        offs.append(offs[-1] + n // 2)
    return (nx, ny, origin, extent, sp, pad), np.array(offs, dtype=np.int32), np.array(vals, dtype=np.float64)


def read_csr_volume(path):
    """The binary CSR dump of CompressedVolume::save_csr."""
    b = open(path, "rb").read()
    assert b[:8] == b"VOCSR001"
    nx, ny, pad = struct.unpack_from("<3i", b, 8)
    geo = struct.unpack_from("<7d", b, 20)
    (nseg,) = struct.unpack_from("<q", b, 76)
    offs = np.frombuffer(b, dtype="<i4", count=nx * ny + 1, offset=84).copy()
    z = np.frombuffer(b, dtype="<f8", count=2 * nseg, offset=84 + 4 * (nx * ny + 1)).copy()
    return (nx, ny, geo[0:3], geo[3:6], geo[6], pad), offs, z


def read_obj(path):
    nv = nf = 0
    verts = []
    faces = []
    for line in open(path):
        if line.startswith("v "):
            nv += 1
            verts.append(tuple(float(t) for t in line.split()[1:4]))
        elif line.startswith("f "):
            nf += 1
            faces.append(tuple(int(t) for t in line.split()[1:]))
    return verts, faces
