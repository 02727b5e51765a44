"""ctypes front end of the CPU oracles.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, and only as the checker. Two libraries:

* ``_build/libvo_oracle.so``: plain-C restatement of the reference algorithm
  (vo_oracle.c), built on every machine by ``make oracle``.
* ``_ref/libvor3d_ref.so``: the reference's own vor3d sources compiled
  unmodified with the project's Eigen/TBB shims (``make ref``); present only
  where the reference source tree exists.

Volumes are exchanged as numpy CSR: ``offs`` int32[nx*ny+1] (in segments) and
``z`` float64[2*nseg].
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libvo_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libvor3d_ref.so")
REF2D_SO = os.path.join(HERE, "_ref", "libvor2d_ref.so")
# the package's input generator built from the same source (make oracle), so that the CPU baseline
# makes its inputs without loading a product library
SYNTH_SO = os.path.join(HERE, "_build", "libvo_synth.so")

OPS = {"dilation": 0, "erosion": 1, "opening": 2, "closing": 3}


class OracleError(RuntimeError):
    pass


class _Grid(C.Structure):
    _fields_ = [
        ("nx", C.c_int),
        ("ny", C.c_int),
        ("origin", C.c_double * 3),
        ("extent", C.c_double * 3),
        ("spacing", C.c_double),
        ("padding", C.c_int),
    ]


class _Csr(C.Structure):
    _fields_ = [("offs", C.POINTER(C.c_int32)), ("z", C.POINTER(C.c_double))]


@dataclass
class Grid:
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


def build(ref: bool | None = None) -> None:
    """Builds the oracle (always) and the reference library (when its sources exist)."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    if ref is None or ref:
        # build_ref.sh knows where the reference sources live and does nothing without them
        subprocess.run(["sh", os.path.join(HERE, "build_ref.sh")], check=True)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build(ref=False)
        L = C.CDLL(ORACLE_SO)
        G, V = C.POINTER(_Grid), C.POINTER(_Csr)
        L.vo_or_dilate.argtypes = [G, V, C.c_double, C.c_int, V, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.vo_or_dilate_brute.argtypes = [G, V, C.c_double, C.c_int, V]
        L.vo_or_morph.argtypes = [C.c_int, C.c_int, G, V, C.c_double, C.c_int, V]
        L.vo_or_xor_volume.argtypes = [G, V, V]
        L.vo_or_xor_volume.restype = C.c_double
        L.vo_or_get_volume.argtypes = [G, V]
        L.vo_or_get_volume.restype = C.c_double
        L.vo_or_dilate_columns.argtypes = [G, V, C.c_double, C.POINTER(C.c_int32), C.c_int, C.c_int, V]
        L.vo_or_morph_columns.argtypes = [C.c_int, G, V, C.c_double, C.POINTER(C.c_int32), C.c_int, C.c_int, V]
        L.vo_or_image_morph.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                        C.c_double, C.POINTER(C.POINTER(C.c_int32)),
                                        C.POINTER(C.POINTER(C.c_int32))]
        L.vo_or_image_morph_f64.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int32),
                                            C.POINTER(C.c_double), C.c_double, C.POINTER(C.POINTER(C.c_int32)),
                                            C.POINTER(C.POINTER(C.c_double))]
        L.vo_or_pass1_pieces.argtypes = [G, V, C.c_double, C.c_int]
        L.vo_or_pass1_pieces.restype = C.c_int64
        L.vo_or_dexelize.argtypes = [C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_int32), C.c_int,
                                     C.POINTER(C.c_double), C.c_int, C.c_int, G, V]
        L.vo_or_free.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def reflib():
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            raise OracleError("reference library not built (oracle/_ref); needs the reference sources")
        L = C.CDLL(REF_SO)
        pd, pi = C.POINTER(C.c_double), C.POINTER(C.c_int32)
        L.ref_morph.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, pd, pd, C.c_double, C.c_int, pi, pd,
                                C.c_double, C.c_int, C.POINTER(pi), C.POINTER(pd), C.POINTER(C.c_int),
                                C.POINTER(C.c_int), pd, pd, pd]
        L.ref_xor_volume.argtypes = [C.c_int, C.c_int, pd, pd, C.c_double, C.c_int, pi, pd, pi, pd]
        L.ref_xor_volume.restype = C.c_double
        L.ref_free.argtypes = [C.c_void_p]
        _ref = L
    return _ref


def _csr_in(offs, z):
    offs = np.ascontiguousarray(offs, dtype=np.int32)
    z = np.ascontiguousarray(z, dtype=np.float64)
    if z.size == 0:
        z = np.zeros(2, dtype=np.float64)
    c = _Csr()
    c.offs = offs.ctypes.data_as(C.POINTER(C.c_int32))
    c.z = z.ctypes.data_as(C.POINTER(C.c_double))
    return c, (offs, z)


def _csr_take(c: _Csr, ncols: int):
    offs = np.ctypeslib.as_array(c.offs, shape=(ncols + 1,)).copy()
    nv = 2 * int(offs[-1])
    z = np.ctypeslib.as_array(c.z, shape=(max(nv, 1),))[:nv].copy()
    lib().vo_or_free(C.cast(c.offs, C.c_void_p))
    lib().vo_or_free(C.cast(c.z, C.c_void_p))
    return offs, z


def _rc(rc, what):
    if rc != 0:
        raise OracleError(f"{what} failed with status {rc}")


def morph(grid: Grid, offs, z, radius: float, op: str = "dilation", method: str = "separable",
          threads: int = 0):
    """Oracle restatement: op in dilation/erosion/opening/closing, method separable/brute."""
    L = lib()
    g = grid.to_c()
    cin, keep = _csr_in(offs, z)
    cout = _Csr()
    m = {"separable": 0, "brute": 1}[method]
    rc = L.vo_or_morph(m, OPS[op], C.byref(g), C.byref(cin), float(radius), threads or os.cpu_count(),
                       C.byref(cout))
    _rc(rc, "vo_or_morph")
    return _csr_take(cout, grid.nx * grid.ny)


def dilate_timed(grid: Grid, offs, z, radius: float, threads: int = 0):
    """Separable dilation returning (offs, z, t1_ms, t2_ms)."""
    L = lib()
    g = grid.to_c()
    cin, keep = _csr_in(offs, z)
    cout = _Csr()
    t1, t2 = C.c_double(), C.c_double()
    rc = L.vo_or_dilate(C.byref(g), C.byref(cin), float(radius), threads or os.cpu_count(), C.byref(cout),
                        C.byref(t1), C.byref(t2))
    _rc(rc, "vo_or_dilate")
    o, zz = _csr_take(cout, grid.nx * grid.ny)
    return o, zz, t1.value, t2.value


def dilate_columns(grid: Grid, offs, z, radius: float, cols, threads: int = 0):
    """Separable dilation of the selected output columns only: returns (offs[len(cols)+1], z)."""
    L = lib()
    cols = np.ascontiguousarray(cols, dtype=np.int32)
    cin, keep = _csr_in(offs, z)
    cout = _Csr()
    rc = L.vo_or_dilate_columns(C.byref(grid.to_c()), C.byref(cin), float(radius),
                                cols.ctypes.data_as(C.POINTER(C.c_int32)), int(cols.size),
                                threads or os.cpu_count(), C.byref(cout))
    _rc(rc, "vo_or_dilate_columns")
    return _csr_take(cout, int(cols.size))


def morph_columns(grid: Grid, offs, z, radius: float, op: str, cols, threads: int = 0):
    """Any op at the selected output columns only: returns (offs[len(cols)+1], z), equal to the
    corresponding columns of morph(grid, offs, z, radius, op)."""
    L = lib()
    cols = np.ascontiguousarray(cols, dtype=np.int32)
    cin, keep = _csr_in(offs, z)
    cout = _Csr()
    rc = L.vo_or_morph_columns(OPS[op], C.byref(grid.to_c()), C.byref(cin), float(radius),
                               cols.ctypes.data_as(C.POINTER(C.c_int32)), int(cols.size),
                               threads or os.cpu_count(), C.byref(cout))
    _rc(rc, "vo_or_morph_columns")
    return _csr_take(cout, int(cols.size))


def pass1_pieces(grid: Grid, offs, z, radius: float, threads: int = 0) -> int:
    cin, keep = _csr_in(offs, z)
    return int(lib().vo_or_pass1_pieces(C.byref(grid.to_c()), C.byref(cin), float(radius),
                                        threads or os.cpu_count()))


def xor_volume(grid: Grid, a, b) -> float:
    ca, k1 = _csr_in(*a)
    cb, k2 = _csr_in(*b)
    return float(lib().vo_or_xor_volume(C.byref(grid.to_c()), C.byref(ca), C.byref(cb)))


def get_volume(grid: Grid, offs, z) -> float:
    c, keep = _csr_in(offs, z)
    return float(lib().vo_or_get_volume(C.byref(grid.to_c()), C.byref(c)))


def dexelize(verts, tris, num_dexels: int = 256, padding: int = 0, spacing: float = 1.0):
    """Oracle restatement of create_dexels; returns (Grid, offs, z)."""
    verts = np.ascontiguousarray(verts, dtype=np.float64).reshape(-1)
    tris = np.ascontiguousarray(tris, dtype=np.int32).reshape(-1)
    sp = C.c_double(spacing)
    g = _Grid()
    out = _Csr()
    rc = lib().vo_or_dexelize(verts.ctypes.data_as(C.POINTER(C.c_double)), verts.size // 3,
                              tris.ctypes.data_as(C.POINTER(C.c_int32)), tris.size // 3, C.byref(sp),
                              int(padding), int(num_dexels), C.byref(g), C.byref(out))
    _rc(rc, "vo_or_dexelize")
    grid = Grid(g.nx, g.ny, tuple(g.origin), tuple(g.extent), g.spacing, g.padding)
    offs, z = _csr_take(out, g.nx * g.ny)
    return grid, offs, z


def ref_morph(grid: Grid, offs, z, radius: float, op: str = "dilation", method: str = "ours",
              threads: int = 1):
    """The reference itself (oracle/_ref). Returns (offs, z, time_ms, t1_ms, t2_ms)."""
    L = reflib()
    offs = np.ascontiguousarray(offs, dtype=np.int32)
    zz = np.ascontiguousarray(z, dtype=np.float64)
    if zz.size == 0:
        zz = np.zeros(2)
    origin = (C.c_double * 3)(*grid.origin)
    extent = (C.c_double * 3)(*grid.extent)
    po, pz = C.POINTER(C.c_int32)(), C.POINTER(C.c_double)()
    onx, ony = C.c_int(), C.c_int()
    tms, t1, t2 = C.c_double(), C.c_double(), C.c_double()
    m = {"ours": 0, "brute_force": 1}[method]
    rc = L.ref_morph(m, OPS[op], grid.nx, grid.ny, origin, extent, float(grid.spacing), int(grid.padding),
                     offs.ctypes.data_as(C.POINTER(C.c_int32)), zz.ctypes.data_as(C.POINTER(C.c_double)),
                     float(radius), int(threads), C.byref(po), C.byref(pz), C.byref(onx), C.byref(ony),
                     C.byref(tms), C.byref(t1), C.byref(t2))
    _rc(rc, "ref_morph")
    n = onx.value * ony.value
    o = np.ctypeslib.as_array(po, shape=(n + 1,)).copy()
    nv = 2 * int(o[-1])
    zo = np.ctypeslib.as_array(pz, shape=(max(nv, 1),))[:nv].copy()
    L.ref_free(C.cast(po, C.c_void_p))
    L.ref_free(C.cast(pz, C.c_void_p))
    return o, zo, tms.value, t1.value, t2.value


IMAGE_OPS = {"dilate": 0, "erode": 1, "open": 2, "close": 3}


def _take_i32(p_offs, p_ev, height, free):
    offs = np.ctypeslib.as_array(p_offs, shape=(height + 1,)).copy()
    n = int(offs[-1])
    ev = np.ctypeslib.as_array(p_ev, shape=(max(n, 1),))[:n].copy()
    free(C.cast(p_offs, C.c_void_p))
    free(C.cast(p_ev, C.c_void_p))
    return offs, ev


def image_morph(width: int, height: int, offs, events, radius: float, op: str = "dilate"):
    """2D image morphology (src/vor2d CompressedImage), restated: returns (offs, events)."""
    offs = np.ascontiguousarray(offs, dtype=np.int32)
    ev = np.ascontiguousarray(events, dtype=np.int32)
    if ev.size == 0:
        ev = np.zeros(1, np.int32)
    po, pe = C.POINTER(C.c_int32)(), C.POINTER(C.c_int32)()
    rc = lib().vo_or_image_morph(IMAGE_OPS[op], int(width), int(height), offs.ctypes.data_as(C.POINTER(C.c_int32)),
                                 ev.ctypes.data_as(C.POINTER(C.c_int32)), float(radius), C.byref(po), C.byref(pe))
    _rc(rc, "vo_or_image_morph")
    return _take_i32(po, pe, height, lib().vo_or_free)


def _take_f64(p_offs, p_ev, height, free):
    offs = np.ctypeslib.as_array(p_offs, shape=(height + 1,)).copy()
    n = int(offs[-1])
    ev = np.ctypeslib.as_array(p_ev, shape=(max(n, 1),))[:n].copy()
    free(C.cast(p_offs, C.c_void_p))
    free(C.cast(p_ev, C.c_void_p))
    return offs, ev


def image_morph_f64(width: int, height: int, offs, events, radius: float, op: str = "dilate"):
    """The FP64 twin (DoubleCompressedImage), restated: returns (offs, events)."""
    offs = np.ascontiguousarray(offs, dtype=np.int32)
    ev = np.ascontiguousarray(events, dtype=np.float64)
    if ev.size == 0:
        ev = np.zeros(1)
    po, pe = C.POINTER(C.c_int32)(), C.POINTER(C.c_double)()
    rc = lib().vo_or_image_morph_f64(IMAGE_OPS[op], int(width), int(height), offs.ctypes.data_as(C.POINTER(C.c_int32)),
                                     ev.ctypes.data_as(C.POINTER(C.c_double)), float(radius), C.byref(po), C.byref(pe))
    _rc(rc, "vo_or_image_morph_f64")
    return _take_f64(po, pe, height, lib().vo_or_free)


def ref_image_morph_f64(width: int, height: int, offs, events, radius: float, op: str = "dilate"):
    """The reference's own DoubleCompressedImage (oracle/_ref/libvor2d_ref.so)."""
    L = C.CDLL(REF2D_SO)
    L.ref2d_morph_f64.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int32), C.POINTER(C.c_double),
                                  C.c_double, C.POINTER(C.POINTER(C.c_int32)), C.POINTER(C.POINTER(C.c_double))]
    L.ref2d_free.argtypes = [C.c_void_p]
    offs = np.ascontiguousarray(offs, dtype=np.int32)
    ev = np.ascontiguousarray(events, dtype=np.float64)
    if ev.size == 0:
        ev = np.zeros(1)
    po, pe = C.POINTER(C.c_int32)(), C.POINTER(C.c_double)()
    rc = L.ref2d_morph_f64(IMAGE_OPS[op], int(width), int(height), offs.ctypes.data_as(C.POINTER(C.c_int32)),
                           ev.ctypes.data_as(C.POINTER(C.c_double)), float(radius), C.byref(po), C.byref(pe))
    _rc(rc, "ref2d_morph_f64")
    return _take_f64(po, pe, height, L.ref2d_free)


def ref2d_available() -> bool:
    return os.path.exists(REF2D_SO)


def ref_image_morph(width: int, height: int, offs, events, radius: float, op: str = "dilate"):
    """The reference's own CompressedImage (oracle/_ref/libvor2d_ref.so): returns (offs, events)."""
    L = C.CDLL(REF2D_SO)
    L.ref2d_morph.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_double,
                              C.POINTER(C.POINTER(C.c_int32)), C.POINTER(C.POINTER(C.c_int32))]
    L.ref2d_free.argtypes = [C.c_void_p]
    offs = np.ascontiguousarray(offs, dtype=np.int32)
    ev = np.ascontiguousarray(events, dtype=np.int32)
    if ev.size == 0:
        ev = np.zeros(1, np.int32)
    po, pe = C.POINTER(C.c_int32)(), C.POINTER(C.c_int32)()
    rc = L.ref2d_morph(IMAGE_OPS[op], int(width), int(height), offs.ctypes.data_as(C.POINTER(C.c_int32)),
                       ev.ctypes.data_as(C.POINTER(C.c_int32)), float(radius), C.byref(po), C.byref(pe))
    _rc(rc, "ref2d_morph")
    return _take_i32(po, pe, height, L.ref2d_free)


def compare(a, b, tol: float = 1e-9):
    """Column-by-column comparison of two CSR volumes.

    Returns dict(count_mismatch=#columns whose segment counts differ,
    max_err=max endpoint |diff| over columns with equal counts, bad_columns=list)."""
    oa, za = a
    ob, zb = b
    oa = np.asarray(oa)
    ob = np.asarray(ob)
    if oa.shape != ob.shape:
        raise ValueError("grids differ")
    ca = np.diff(oa)
    cb = np.diff(ob)
    bad = np.nonzero(ca != cb)[0]
    same = ca == cb
    max_err = 0.0
    if za.size and zb.size and same.any():
        # gather endpoints of columns with equal counts
        reps = np.repeat(same, 2 * ca)
        ea = np.asarray(za)[reps]
        rb = np.repeat(same, 2 * cb)
        eb = np.asarray(zb)[rb]
        if ea.size:
            max_err = float(np.max(np.abs(ea - eb)))
    err_cols = []
    if max_err > tol:
        idx = np.nonzero(same)[0]
        for c in idx:
            sa = za[2 * oa[c]:2 * oa[c + 1]]
            sb = zb[2 * ob[c]:2 * ob[c + 1]]
            if sa.size and np.max(np.abs(sa - sb)) > tol:
                err_cols.append(int(c))
                if len(err_cols) > 20:
                    break
    return {"count_mismatch": int(bad.size), "max_err": max_err, "bad_columns": bad[:20].tolist(),
            "err_columns": err_cols}
