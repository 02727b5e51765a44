"""The C-ABI library without a GPU: it loads, exports every function the
public header declares, its host utilities are deterministic, and device
entry points fail cleanly (no CPU fallback) when no sm_103 device exists."""
from __future__ import annotations

import glob
import hashlib
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def header_functions(name: str | None = None):
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", name or "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"\b(vo_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_header_declares_the_boundary():
    names = header_functions()
    for required in ["vo_create", "vo_destroy", "vo_volume_upload", "vo_volume_download", "vo_volume_info",
                     "vo_morph", "vo_morph_batched", "vo_dexelize", "vo_last_error", "vo_xor_volume"]:
        assert required in names


def test_library_exports_every_declared_symbol(vo):
    # voroffset_gpu.h -> libvoroffset_gpu.so, voroffset_synth.h -> libvoroffset_synth.so
    for header, L, path in (("voroffset_gpu.h", vo.lib(), vo.LIB_PATH),
                            ("voroffset_synth.h", vo.synth_lib(), vo.SYNTH_LIB_PATH)):
        missing = [n for n in header_functions(header) if not hasattr(L, n)]
        assert not missing, f"symbols declared in {header} but not exported: {missing}"
        out = os.popen(f"nm -D --defined-only {path}").read()
        exported = set(re.findall(r" T (vo_[a-z0-9_]+)", out))
        assert set(header_functions(header)) <= exported


def test_gpu_library_holds_no_input_generator(vo):
    out = os.popen(f"nm -D --defined-only {vo.LIB_PATH}").read()
    assert "vo_synth_volume" not in out and "vo_synth_torus" not in out


def test_python_mirror_covers_header(vo):
    assert set(header_functions("voroffset_gpu.h")) <= set(vo.SIGNATURES)
    assert set(header_functions("voroffset_synth.h")) <= set(vo.SYNTH_SIGNATURES)


def test_synth_is_deterministic(vo):
    spec = vo.SynthSpec(64, n_spheres=20, n_cyl=10, seed=123)
    a = vo.synth_volume(spec)
    b = vo.synth_volume(spec)
    assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])
    c = vo.synth_volume(vo.SynthSpec(64, n_spheres=20, n_cyl=10, seed=124))
    assert not np.array_equal(a[2], c[2])
    # columns are sorted and disjoint, within [0, zmax]
    g, offs, z = a
    for col in range(g.ncols):
        s = z[2 * offs[col]:2 * offs[col + 1]]
        assert np.all(np.diff(s) >= 0)
        if s.size:
            assert s[0] >= 0 and s[-1] <= 64
        assert np.all(s[2::2] > s[1:-1:2])


def test_synth_fixture_hash_is_stable(vo):
    # pins the generator across machines (x86 container vs aarch64 GPU host)
    g, offs, z = vo.synth_volume(vo.SynthSpec(48, n_spheres=24, s_rmin=3, s_rmax=14, seed=11))
    d = np.load(os.path.join(ROOT, "tests", "golden", "spheres48_r5.npz"))
    assert np.array_equal(offs, d["offs"]) and np.array_equal(z, d["z"])


def test_torus_is_watertight(vo):
    verts, tris = vo.synth_torus(32, 12, seed=3)
    edges = {}
    for t in tris:
        for a, b in ((t[0], t[1]), (t[1], t[2]), (t[2], t[0])):
            edges[(a, b)] = edges.get((a, b), 0) + 1
    for (a, b), n in edges.items():
        assert n == 1 and edges.get((b, a)) == 1


def test_device_calls_fail_cleanly_without_gpu(vo):
    import ctypes as C
    n = C.c_int()
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(vo.GpuError) as e:
        vo.Context(0)
    assert e.value.code == vo.VO_ENODEV
