"""Python front end of libvoroffset_gpu.so (the C ABI in include/voroffset_gpu.h).

A thin ctypes layer used by tests and bench.py; the product is the shared
library and its C ABI. Mirrors the reference's method layer
(src/vor3d/Voronoi.h:13-44): ``Context.morph(volume, "dilation", r)`` is
``VoronoiMorpho::dilation``, with erosion / opening / closing chained as
app/cli3d/offset3d.cpp:116-136 does. There is no CPU fallback: when the
library or an sm_103 device is missing, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libvoroffset_gpu.so")

VO_OK, VO_EINVAL, VO_ENOMEM, VO_ECUDA, VO_ERADIUS, VO_ERANGE, VO_ENODEV, VO_ETIMEOUT, VO_EINTERNAL = (
    0, -1, -2, -3, -4, -5, -6, -7, -8)
OPS = {"dilation": 0, "erosion": 1, "opening": 2, "closing": 3}
METHODS = {"separable": 0, "brute": 1, "fast": 2, "envelope": 3}
STATUS = {0: "VO_OK", -1: "VO_EINVAL", -2: "VO_ENOMEM", -3: "VO_ECUDA", -4: "VO_ERADIUS",
          -5: "VO_ERANGE", -6: "VO_ENODEV", -7: "VO_ETIMEOUT", -8: "VO_EINTERNAL"}


class GpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class _Grid(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("origin", C.c_double * 3),
                ("extent", C.c_double * 3), ("spacing", C.c_double), ("padding", C.c_int32)]


class _Timings(C.Structure):
    _fields_ = [("total_ms", C.c_double), ("pass1_ms", C.c_double), ("pass2_ms", C.c_double),
                ("in_segments", C.c_int64), ("mid_pieces", C.c_int64), ("out_segments", C.c_int64),
                ("kernel_launches", C.c_int32), ("overflow_columns", C.c_int32),
                ("kernel_ms", C.c_double * 4)]


class _SynthParams(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("zmax", C.c_double), ("n_spheres", C.c_int32),
                ("sphere_dist", C.c_int32), ("s_rmin", C.c_double), ("s_rmax", C.c_double),
                ("s_median", C.c_double), ("s_sigma", C.c_double), ("n_cyl", C.c_int32),
                ("c_rmin", C.c_double), ("c_rmax", C.c_double), ("seed", C.c_uint64)]


class _BatchStats(C.Structure):
    _fields_ = [("slot_bytes", C.c_int64), ("tiles", C.c_int32), ("tile_rows", C.c_int32),
                ("union_cap", C.c_int32), ("persistent", C.c_int32), ("regs", C.c_int32), ("graph_nodes", C.c_int32), ("graph_kernels", C.c_int32), ("learned", C.c_int32),
                ("reruns", C.c_int32), ("rerun_first", C.c_int32), ("rerun_cause", C.c_int32), ("spill_peak", C.c_double),
                ("spill_peak_round", C.c_int32), ("plan_ms", C.c_double), ("tune_ms", C.c_double * 4)]


SIZER_FEATURES = 16
SIZER_OUTPUTS = 3


@dataclass
class Grid:
    """CompressedVolume geometry (CompressedVolumeBase.h:17-21); origin already padded."""
    nx: int
    ny: int
    origin: tuple = (0.0, 0.0, 0.0)
    extent: tuple = (0.0, 0.0, 0.0)
    spacing: float = 1.0
    padding: int = 0

    def to_c(self) -> _Grid:
        g = _Grid()
        g.nx, g.ny = int(self.nx), int(self.ny)
        g.origin[:] = [float(v) for v in self.origin]
        g.extent[:] = [float(v) for v in self.extent]
        g.spacing = float(self.spacing)
        g.padding = int(self.padding)
        return g

    @staticmethod
    def from_c(g: _Grid) -> "Grid":
        return Grid(g.nx, g.ny, tuple(g.origin), tuple(g.extent), g.spacing, g.padding)

    @property
    def ncols(self) -> int:
        return self.nx * self.ny


_lib = None

# Every function of include/voroffset_gpu.h with its ctypes signature.
_P = C.c_void_p
SIGNATURES = {
    "vo_create": (C.c_int, [C.POINTER(_P), C.c_int]),
    "vo_destroy": (None, [_P]),
    "vo_last_error": (C.c_char_p, [_P]),
    "vo_stream": (_P, [_P]),
    "vo_sync": (C.c_int, [_P]),
    "vo_volume_upload": (C.c_int, [_P, C.POINTER(_Grid), C.POINTER(C.c_int32), C.POINTER(C.c_double),
                                   C.POINTER(_P)]),
    "vo_volume_upload_async": (C.c_int, [_P, C.POINTER(_Grid), C.POINTER(C.c_int32), C.POINTER(C.c_double),
                                   C.POINTER(_P)]),
    "vo_volume_info": (C.c_int, [_P, _P, C.POINTER(_Grid), C.POINTER(C.c_int64)]),
    "vo_volume_download": (C.c_int, [_P, _P, C.POINTER(C.c_int32), C.POINTER(C.c_double)]),
    "vo_volume_download_async": (C.c_int, [_P, _P, C.POINTER(C.c_int32), C.POINTER(C.c_double)]),
    "vo_volume_device_ptrs": (C.c_int, [_P, _P, C.POINTER(_P), C.POINTER(_P)]),
    "vo_volume_free": (None, [_P, _P]),
    "vo_morph": (C.c_int, [_P, C.c_int, C.c_int, C.c_double, _P, C.POINTER(_P), C.POINTER(_Timings)]),
    "vo_morph_batched": (C.c_int, [_P, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_int,
                                   C.POINTER(_P), C.POINTER(_P), C.POINTER(_Timings)]),
    "vo_dexelize": (C.c_int, [_P, C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_int32), C.c_int,
                              C.POINTER(C.c_double), C.c_int, C.c_int, C.POINTER(_P)]),
    "vo_dexelize_odd_columns": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "vo_xor_volume": (C.c_int, [_P, _P, _P, C.POINTER(C.c_double)]),
    "vo_volume_measure": (C.c_int, [_P, _P, C.POINTER(C.c_int64), C.POINTER(C.c_double)]),
    "vo_image_morph": (C.c_int, [_P, C.c_int, C.c_double, C.c_int, C.c_int, C.POINTER(C.c_int32),
                                 C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_int64]),
    "vo_image_morph_f64": (C.c_int, [_P, C.c_int, C.c_double, C.c_int, C.c_int, C.POINTER(C.c_int32),
                                     C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_double), C.c_int64]),
    "vo_xor_volume_noalloc": (C.c_int, [C.POINTER(_Grid), _P, _P, _P, _P, _P, C.POINTER(C.c_double)]),
    "vo_batch_create": (C.c_int, [_P, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_int,
                                  C.POINTER(_P), C.POINTER(_P)]),
    "vo_batch_run": (C.c_int, [_P, _P, C.POINTER(_Timings)]),
    "vo_batch_outputs": (C.c_int, [_P, _P, C.POINTER(_P)]),
    "vo_batch_stats_get": (C.c_int, [_P, _P, C.POINTER(_BatchStats)]),
    "vo_batch_destroy": (None, [_P, _P]),
    "vo_sizer_create": (C.c_int, [_P, C.c_uint64, C.POINTER(_P)]),
    "vo_sizer_destroy": (None, [_P, _P]),
    "vo_sizer_num_params": (C.c_int, []),
    "vo_sizer_set_params": (C.c_int, [_P, _P, C.POINTER(C.c_float), C.c_int]),
    "vo_sizer_get_params": (C.c_int, [_P, _P, C.POINTER(C.c_float), C.c_int]),
    "vo_sizer_tile_features": (C.c_int, [_P, _P, C.c_double, C.POINTER(C.c_float), C.POINTER(C.c_int)]),
    "vo_sizer_tile_targets": (C.c_int, [_P, _P, _P, C.c_double, C.POINTER(C.c_float), C.POINTER(C.c_int)]),
    "vo_sizer_forward": (C.c_int, [_P, _P, C.POINTER(C.c_float), C.c_int, C.POINTER(C.c_float)]),
    "vo_sizer_gradients": (C.c_int, [_P, _P, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int,
                                     C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "vo_sizer_train": (C.c_int, [_P, _P, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int, C.c_int,
                                 C.c_float, C.POINTER(C.c_float)]),
    "vo_set_sizer": (C.c_int, [_P, _P]),
}

# Every function of include/voroffset_synth.h (the host-only input generator,
# libvoroffset_synth.so) with its ctypes signature.
SYNTH_LIB_PATH = os.path.join(PKG, "libvoroffset_synth.so")
SYNTH_SIGNATURES = {
    "vo_synth_volume": (C.c_int, [C.POINTER(_SynthParams), C.POINTER(C.c_int32),
                                  C.POINTER(C.POINTER(C.c_double)), C.POINTER(C.c_int64)]),
    "vo_synth_torus": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_uint64,
                                 C.POINTER(C.POINTER(C.c_double)), C.POINTER(C.c_int),
                                 C.POINTER(C.POINTER(C.c_int32)), C.POINTER(C.c_int)]),
    "vo_host_free": (None, [_P]),
}
_synth = {}


def synth_lib(path: str | None = None) -> C.CDLL:
    """Loads the input generator: libvoroffset_synth.so, or the same source built at `path`."""
    path = path or SYNTH_LIB_PATH
    if path not in _synth:
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: run `python -m voroffset_gb300.build`")
        L = C.CDLL(path)
        for name, (res, args) in SYNTH_SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _synth[path] = L
    return _synth[path]


def lib(build_if_missing: bool = False) -> C.CDLL:
    """Loads libvoroffset_gpu.so; raises if it was not built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            if build_if_missing:
                from . import build as _b
                _b.build()
            else:
                raise RuntimeError(f"{LIB_PATH} is missing: run `python -m voroffset_gb300.build`")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _i32p(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def _f64p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Volume:
    """A device-resident CSR volume owned by a Context."""

    def __init__(self, ctx: "Context", handle: int):
        self.ctx = ctx
        self.handle = handle
        g = _Grid()
        n = C.c_int64()
        lib().vo_volume_info(ctx.handle, handle, C.byref(g), C.byref(n))
        self.grid = Grid.from_c(g)
        self.nseg = int(n.value)

    def download(self):
        return self.ctx.download(self)

    def device_ptrs(self):
        po, pz = C.c_void_p(), C.c_void_p()
        lib().vo_volume_device_ptrs(self.ctx.handle, self.handle, C.byref(po), C.byref(pz))
        return po.value, pz.value

    def free(self):
        if self.handle:
            lib().vo_volume_free(self.ctx.handle, self.handle)
            self.handle = None

    def __del__(self):
        try:
            if self.handle and self.ctx.handle:
                self.free()
        except Exception:
            pass


class Context:
    """vo_ctx: one CUDA stream on one device."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        rc = lib().vo_create(C.byref(h), int(device))
        if rc != VO_OK:
            raise GpuError(rc, "vo_create failed (an sm_103 device is required)")
        self.handle = h.value

    def _check(self, rc: int, what: str):
        if rc != VO_OK:
            msg = lib().vo_last_error(self.handle)
            raise GpuError(rc, f"{what}: {msg.decode() if msg else ''}")

    @property
    def stream(self) -> int:
        return lib().vo_stream(self.handle)

    def sync(self):
        self._check(lib().vo_sync(self.handle), "vo_sync")

    def close(self):
        if self.handle:
            lib().vo_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def upload(self, grid: Grid, offs, z) -> Volume:
        offs = np.ascontiguousarray(offs, dtype=np.int32)
        z = np.ascontiguousarray(z, dtype=np.float64)
        if offs.size != grid.ncols + 1:
            raise ValueError("offs must have nx*ny+1 entries")
        zz = z if z.size else np.zeros(2)
        h = C.c_void_p()
        g = grid.to_c()
        self._check(lib().vo_volume_upload(self.handle, C.byref(g), _i32p(offs), _f64p(zz), C.byref(h)),
                    "vo_volume_upload")
        return Volume(self, h.value)

    def upload_async(self, grid: Grid, offs, z) -> Volume:
        """vo_volume_upload_async: the copy runs on the context's copy stream. offs and z must be
        page-locked (e.g. numpy views of pinned torch tensors), contiguous, and kept unchanged (and
        alive) until sync() or a call that returns results."""
        if offs.dtype != np.int32 or z.dtype != np.float64 or not offs.flags.c_contiguous or \
                not z.flags.c_contiguous:
            raise ValueError("upload_async needs contiguous int32 offsets and float64 pairs")
        if offs.size != grid.ncols + 1:
            raise ValueError("offs must have nx*ny+1 entries")
        h = C.c_void_p()
        g = grid.to_c()
        self._check(lib().vo_volume_upload_async(self.handle, C.byref(g), _i32p(offs), _f64p(z), C.byref(h)),
                    "vo_volume_upload_async")
        return Volume(self, h.value)

    def download_async(self, v: Volume, offs_buf, z_buf):
        """vo_volume_download_async into page-locked caller buffers; they hold the volume after
        sync(). Returns the (offsets, values) counts that will be written."""
        if offs_buf.size < v.grid.ncols + 1 or z_buf.size < 2 * v.nseg:
            raise ValueError("download buffers too small")
        self._check(lib().vo_volume_download_async(self.handle, v.handle, _i32p(offs_buf), _f64p(z_buf)),
                    "vo_volume_download_async")
        return v.grid.ncols + 1, 2 * v.nseg

    def download(self, v: Volume):
        offs = np.empty(v.grid.ncols + 1, dtype=np.int32)
        z = np.empty(max(2 * v.nseg, 2), dtype=np.float64)
        self._check(lib().vo_volume_download(self.handle, v.handle, _i32p(offs), _f64p(z)),
                    "vo_volume_download")
        return offs, z[:2 * v.nseg]

    def download_into(self, v: Volume, offs_buf, z_buf):
        """Downloads into caller buffers (e.g. pinned host memory) sized >= the volume."""
        if offs_buf.size < v.grid.ncols + 1 or z_buf.size < 2 * v.nseg:
            raise ValueError("download buffers too small")
        self._check(lib().vo_volume_download(self.handle, v.handle, _i32p(offs_buf), _f64p(z_buf)),
                    "vo_volume_download")
        return v.grid.ncols + 1, 2 * v.nseg

    def morph(self, v: Volume, op: str = "dilation", radius: float = 8.0, method: str = "separable"):
        out = C.c_void_p()
        t = _Timings()
        self._check(lib().vo_morph(self.handle, OPS[op], METHODS[method], float(radius), v.handle,
                                   C.byref(out), C.byref(t)), "vo_morph")
        return Volume(self, out.value), timings_dict(t)

    def morph_batched(self, vols, ops, radii, method: str = "separable"):
        n = len(vols)
        ops_a = (C.c_int * n)(*[OPS[o] for o in ops])
        rad_a = (C.c_double * n)(*[float(r) for r in radii])
        ins = (C.c_void_p * n)(*[v.handle for v in vols])
        outs = (C.c_void_p * n)()
        t = _Timings()
        self._check(lib().vo_morph_batched(self.handle, n, ops_a, rad_a, METHODS[method], ins, outs,
                                           C.byref(t)), "vo_morph_batched")
        return [Volume(self, outs[i]) for i in range(n)], timings_dict(t)

    def batch(self, vols, ops, radii, method: str = "fast") -> "Batch":
        """A batch plan (vo_batch_create): planned, sized, tuned and captured once, replayed by run()."""
        n = len(vols)
        ops_a = (C.c_int * n)(*[OPS[o] for o in ops])
        rad_a = (C.c_double * n)(*[float(r) for r in radii])
        ins = (C.c_void_p * n)(*[v.handle for v in vols])
        out = C.c_void_p()
        self._check(lib().vo_batch_create(self.handle, n, ops_a, rad_a, METHODS[method], ins, C.byref(out)),
                    "vo_batch_create")
        return Batch(self, out.value, list(vols))

    def sizer(self, seed: int = 1) -> "Sizer":
        out = C.c_void_p()
        self._check(lib().vo_sizer_create(self.handle, int(seed), C.byref(out)), "vo_sizer_create")
        return Sizer(self, out.value)

    def set_sizer(self, s: "Sizer | None"):
        self._check(lib().vo_set_sizer(self.handle, s.handle if s is not None else None), "vo_set_sizer")

    def dexelize(self, verts, tris, num_dexels: int = 256, padding: int = 0, spacing: float = 1.0):
        verts = np.ascontiguousarray(verts, dtype=np.float64).reshape(-1)
        tris = np.ascontiguousarray(tris, dtype=np.int32).reshape(-1)
        sp = C.c_double(spacing)
        out = C.c_void_p()
        self._check(lib().vo_dexelize(self.handle, _f64p(verts), verts.size // 3, _i32p(tris), tris.size // 3,
                                      C.byref(sp), int(padding), int(num_dexels), C.byref(out)),
                    "vo_dexelize")
        return Volume(self, out.value)

    def dexelize_odd_columns(self) -> int:
        """Columns of the last dexelize whose ray met the mesh an odd number of times (last hit dropped)."""
        n = C.c_int64()
        self._check(lib().vo_dexelize_odd_columns(self.handle, C.byref(n)), "vo_dexelize_odd_columns")
        return int(n.value)

    def image_morph(self, width: int, height: int, row_offs, events, radius: float, op: str = "dilation"):
        """2D image morphology (CompressedImage): returns (row_offs, events) of the result."""
        ro = np.ascontiguousarray(row_offs, dtype=np.int32)
        ev = np.ascontiguousarray(events, dtype=np.int32)
        if ev.size == 0:
            ev = np.zeros(1, np.int32)
        out_o = np.zeros(height + 1, np.int32)
        cap = max(16, 2 * int(ro[-1]) + 2 * height)
        while True:
            out_e = np.zeros(cap, np.int32)
            rc = lib().vo_image_morph(self.handle, OPS[op], float(radius), int(width), int(height), _i32p(ro),
                                      _i32p(ev), _i32p(out_o), _i32p(out_e), cap)
            if rc == VO_ERANGE and int(out_o[-1]) > cap:
                cap = int(out_o[-1])
                continue
            self._check(rc, "vo_image_morph")
            return out_o, out_e[:int(out_o[-1])].copy()

    def image_morph_f64(self, width: int, height: int, row_offs, events, radius: float, op: str = "dilation"):
        """The FP64 twin (DoubleCompressedImage): returns (row_offs, events) of the result."""
        ro = np.ascontiguousarray(row_offs, dtype=np.int32)
        ev = np.ascontiguousarray(events, dtype=np.float64)
        if ev.size == 0:
            ev = np.zeros(1)
        out_o = np.zeros(height + 1, np.int32)
        cap = max(16, 2 * int(ro[-1]) + 4 * height)
        while True:
            out_e = np.zeros(cap)
            rc = lib().vo_image_morph_f64(self.handle, OPS[op], float(radius), int(width), int(height), _i32p(ro),
                                          _f64p(ev), _i32p(out_o), _f64p(out_e), cap)
            if rc == VO_ERANGE and int(out_o[-1]) > cap:
                cap = int(out_o[-1])
                continue
            self._check(rc, "vo_image_morph_f64")
            return out_o, out_e[:int(out_o[-1])].copy()

    def measure(self, v: Volume):
        """(numSegments, get_volume) of a volume, reduced on the device."""
        n, vol = C.c_int64(), C.c_double()
        self._check(lib().vo_volume_measure(self.handle, v.handle, C.byref(n), C.byref(vol)), "vo_volume_measure")
        return int(n.value), float(vol.value)

    def xor_volume(self, a: Volume, b: Volume) -> float:
        r = C.c_double()
        self._check(lib().vo_xor_volume(self.handle, a.handle, b.handle, C.byref(r)), "vo_xor_volume")
        return float(r.value)


class Batch:
    """A captured batch plan; keeps its input volumes alive."""

    def __init__(self, ctx: Context, handle: int, inputs):
        self.ctx, self.handle, self._inputs = ctx, handle, inputs

    def run(self) -> dict:
        t = _Timings()
        self.ctx._check(lib().vo_batch_run(self.ctx.handle, self.handle, C.byref(t)), "vo_batch_run")
        return timings_dict(t)

    def outputs(self):
        n = len(self._inputs)
        outs = (C.c_void_p * max(n, 1))()
        self.ctx._check(lib().vo_batch_outputs(self.ctx.handle, self.handle, outs), "vo_batch_outputs")
        return [Volume(self.ctx, outs[i]) for i in range(n)]

    def stats(self) -> dict:
        s = _BatchStats()
        self.ctx._check(lib().vo_batch_stats_get(self.ctx.handle, self.handle, C.byref(s)), "vo_batch_stats_get")
        d = {k: getattr(s, k) for k, _ in _BatchStats._fields_}
        d["tune_ms"] = list(s.tune_ms)
        return d

    def free(self):
        if self.handle:
            lib().vo_batch_destroy(self.ctx.handle, self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def _f32p(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class Sizer:
    """The learned tile sizer (vo_sizer_*): an MLP trained and evaluated on the device."""

    def __init__(self, ctx: Context, handle: int):
        self.ctx, self.handle = ctx, handle

    @staticmethod
    def num_params() -> int:
        return int(lib().vo_sizer_num_params())

    def params(self) -> np.ndarray:
        p = np.zeros(self.num_params(), np.float32)
        self.ctx._check(lib().vo_sizer_get_params(self.ctx.handle, self.handle, _f32p(p), p.size),
                        "vo_sizer_get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        self.ctx._check(lib().vo_sizer_set_params(self.ctx.handle, self.handle, _f32p(p), p.size),
                        "vo_sizer_set_params")

    def features(self, v: Volume, radius: float) -> np.ndarray:
        n = C.c_int()
        self.ctx._check(lib().vo_sizer_tile_features(self.ctx.handle, v.handle, float(radius), None, C.byref(n)),
                        "vo_sizer_tile_features")
        f = np.zeros((n.value, SIZER_FEATURES), np.float32)
        self.ctx._check(lib().vo_sizer_tile_features(self.ctx.handle, v.handle, float(radius), _f32p(f),
                                                     C.byref(n)), "vo_sizer_tile_features")
        return f

    def targets(self, v: Volume, result: Volume, radius: float) -> np.ndarray:
        g = C.c_int()
        nt = len(self.features(v, radius))
        t = np.zeros((nt, SIZER_OUTPUTS), np.float32)
        self.ctx._check(lib().vo_sizer_tile_targets(self.ctx.handle, v.handle, result.handle, float(radius),
                                                    _f32p(t), C.byref(g)), "vo_sizer_tile_targets")
        return t

    def forward(self, feats) -> np.ndarray:
        feats = np.ascontiguousarray(feats, dtype=np.float32)
        out = np.zeros((len(feats), SIZER_OUTPUTS), np.float32)
        self.ctx._check(lib().vo_sizer_forward(self.ctx.handle, self.handle, _f32p(feats), len(feats),
                                               _f32p(out)), "vo_sizer_forward")
        return out

    def gradients(self, feats, targets):
        feats = np.ascontiguousarray(feats, dtype=np.float32)
        targets = np.ascontiguousarray(targets, dtype=np.float32)
        g = np.zeros(self.num_params(), np.float32)
        loss = C.c_float()
        self.ctx._check(lib().vo_sizer_gradients(self.ctx.handle, self.handle, _f32p(feats), _f32p(targets),
                                                 len(feats), _f32p(g), C.byref(loss)), "vo_sizer_gradients")
        return g, float(loss.value)

    def train(self, feats, targets, steps: int = 500, lr: float = 3e-3) -> float:
        feats = np.ascontiguousarray(feats, dtype=np.float32)
        targets = np.ascontiguousarray(targets, dtype=np.float32)
        loss = C.c_float()
        self.ctx._check(lib().vo_sizer_train(self.ctx.handle, self.handle, _f32p(feats), _f32p(targets),
                                             len(feats), int(steps), float(lr), C.byref(loss)), "vo_sizer_train")
        return float(loss.value)

    def free(self):
        if self.handle:
            lib().vo_sizer_destroy(self.ctx.handle, self.handle)
            self.handle = None


def timings_dict(t: _Timings) -> dict:
    d = {k: getattr(t, k) for k, _ in _Timings._fields_}
    d["kernel_ms"] = list(t.kernel_ms)
    return d


# ---------------------------------------------------------------- host utilities

@dataclass
class SynthSpec:
    """Seeded union of spheres and flat-capped cylinders on an n x n grid, z in [0, zmax]."""
    n: int
    n_spheres: int = 0
    sphere_dist: str = "uniform"  # or "lognormal"
    s_rmin: float = 4.0
    s_rmax: float = 40.0
    s_median: float = 12.0
    s_sigma: float = 0.5
    n_cyl: int = 0
    c_rmin: float = 1.0
    c_rmax: float = 4.0
    seed: int = 1
    zmax: float | None = None
    ny: int | None = None


def synth_volume(spec: SynthSpec, synth: str | None = None):
    """Returns (Grid, offs, z) with spacing 1, origin 0, padding 0, extent (nx, ny, zmax).
    `synth`: path of another build of the generator (default libvoroffset_synth.so)."""
    nx = int(spec.n)
    ny = int(spec.ny or spec.n)
    zmax = float(spec.zmax if spec.zmax is not None else spec.n)
    p = _SynthParams(nx, ny, zmax, int(spec.n_spheres), 1 if spec.sphere_dist == "lognormal" else 0,
                     spec.s_rmin, spec.s_rmax, spec.s_median, spec.s_sigma, int(spec.n_cyl), spec.c_rmin,
                     spec.c_rmax, int(spec.seed) & ((1 << 64) - 1))
    offs = np.zeros(nx * ny + 1, dtype=np.int32)
    pz = C.POINTER(C.c_double)()
    ns = C.c_int64()
    L = synth_lib(synth)
    rc = L.vo_synth_volume(C.byref(p), _i32p(offs), C.byref(pz), C.byref(ns))
    if rc != VO_OK:
        raise GpuError(rc, "vo_synth_volume")
    n2 = 2 * int(ns.value)
    z = np.ctypeslib.as_array(pz, shape=(max(n2, 1),))[:n2].copy()
    L.vo_host_free(C.cast(pz, C.c_void_p))
    grid = Grid(nx, ny, (0.0, 0.0, 0.0), (float(nx), float(ny), zmax), 1.0, 0)
    return grid, offs, z


def synth_torus(nu: int = 256, nv: int = 64, major: float = 0.30, minor: float = 0.10, noise: float = 0.01,
                seed: int = 1):
    pv = C.POINTER(C.c_double)()
    pt = C.POINTER(C.c_int32)()
    nvv, ntt = C.c_int(), C.c_int()
    L = synth_lib()
    rc = L.vo_synth_torus(nu, nv, major, minor, noise, seed, C.byref(pv), C.byref(nvv), C.byref(pt),
                          C.byref(ntt))
    if rc != VO_OK:
        raise GpuError(rc, "vo_synth_torus")
    verts = np.ctypeslib.as_array(pv, shape=(3 * nvv.value,)).copy().reshape(-1, 3)
    tris = np.ctypeslib.as_array(pt, shape=(3 * ntt.value,)).copy().reshape(-1, 3)
    L.vo_host_free(C.cast(pv, C.c_void_p))
    L.vo_host_free(C.cast(pt, C.c_void_p))
    return verts, tris


# Named workloads of the benchmark configurations (sizes and distributions).
def workload_spec(name: str, seed: int = 1) -> SynthSpec:
    """Generator parameters of a named configuration."""
    if name == "spheres1024":
        return SynthSpec(1024, n_spheres=4096, s_rmin=4, s_rmax=40, seed=seed)
    if name == "spheres_cyl2048":
        return SynthSpec(2048, n_spheres=16384, sphere_dist="lognormal", s_median=12, s_sigma=0.5, s_rmin=2,
                         s_rmax=80, n_cyl=2000, c_rmin=1, c_rmax=4, seed=seed)
    if name == "cyl4096":
        return SynthSpec(4096, n_cyl=20000, c_rmin=1.5, c_rmax=3.0, seed=seed)
    raise KeyError(name)


def workload(name: str, seed: int = 1, synth: str | None = None):
    """Synthetic volume for a named configuration: returns (Grid, offs, z)."""
    return synth_volume(workload_spec(name, seed), synth)
