"""Synthetic tissue geometries (seeded) and the host mirror-boundary map.

The reference reads its geometry from files it does not distribute
(wholeventriclewithfibervector.txt, 157layerwithfibervector.txt,
stimulationprofile.cnd; GPU3D.cu:1276,1694, new_11.cu:1296,1723).  These
generators, implemented in C++ behind the C ABI, stand in for them with the
same layout (x-major, z fastest; empty voxels = LQT_EMPTY).
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import _native as N


def _p(a):
    return None if a is None else a.ctypes.data


class VentricleSpec(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("reserved0", C.c_int32),
                ("dx", C.c_double), ("a_out", C.c_double), ("c_out", C.c_double), ("wall", C.c_double),
                ("cx", C.c_double), ("cy", C.c_double), ("z_base", C.c_double), ("endo_frac", C.c_double),
                ("epi_frac", C.c_double), ("island_radius", C.c_double), ("alpha_endo_deg", C.c_double),
                ("alpha_epi_deg", C.c_double), ("stim_radius", C.c_double), ("seed", C.c_uint64)]


def _bind():
    L = N.lib()
    P = C.c_void_p
    L.lqt_geom_sheet.argtypes = [C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_int32, P, P, P]
    L.lqt_geom_sheet.restype = C.c_int
    L.lqt_geom_ventricle.argtypes = [C.POINTER(VentricleSpec), P, P, P, P]
    L.lqt_geom_ventricle.restype = C.c_int
    L.lqt_geom_mirror_map.argtypes = [C.c_int32, C.c_int32, C.c_int32, P, P, P, P, C.POINTER(C.c_int64)]
    L.lqt_geom_mirror_map.restype = C.c_int
    L.lqt_geom_mirror_map_gpu.argtypes = [C.c_int32, C.c_int32, C.c_int32, P, P, P, P, C.POINTER(C.c_int64), P]
    L.lqt_geom_mirror_map_gpu.restype = C.c_int
    return L


@dataclass
class Sheet:
    types: np.ndarray      # (nx+2, ny+2) uint8
    s1_mask: np.ndarray
    s2_mask: np.ndarray


def sheet(nx=600, ny=600, frac_endo=0.30, frac_mid=0.35, s1_cols=3) -> Sheet:
    """2D sheet: nx*ny tissue, bands along x (30% endo / 35% M / 35% epi),
    S1 on the x = 0 edge, S2 on the quadrant x < nx/2, y < ny/2."""
    L = _bind()
    t = np.zeros((nx + 2, ny + 2), np.uint8)
    m1 = np.zeros_like(t)
    m2 = np.zeros_like(t)
    N.check(L.lqt_geom_sheet(nx, ny, frac_endo, frac_mid, s1_cols, _p(t), _p(m1), _p(m2)), "lqt_geom_sheet")
    return Sheet(t, m1, m2)


@dataclass
class Ventricle:
    types: np.ndarray      # (nx, ny, nz) uint8
    fibre: np.ndarray      # (nx, ny, nz, 3) float32
    s1_mask: np.ndarray
    island: np.ndarray     # M-island centre, mm
    spec: VentricleSpec


def ventricle(nx=320, ny=320, nz=420, dx=0.2, a_out=25.0, c_out=62.0, wall=10.0, cx=None, cy=None, z_base=72.0,
              endo_frac=0.3, epi_frac=0.35, island_radius=8.0, alpha_endo=60.0, alpha_epi=-60.0,
              stim_radius=3.0, seed=1234) -> Ventricle:
    """Truncated prolate-ellipsoid shell (default: 320x320x420 at 0.2 mm,
    10 mm wall, about 7M tissue voxels), fibres rotating +60 -> -60 degrees
    from endo to epi, endo/epi by depth with a seeded 8 mm M-cell island,
    apical S1 region."""
    L = _bind()
    sp = VentricleSpec(nx, ny, nz, 0, dx, a_out, c_out, wall, cx if cx is not None else nx * dx / 2,
                       cy if cy is not None else ny * dx / 2, z_base, endo_frac, epi_frac, island_radius, alpha_endo,
                       alpha_epi, stim_radius, seed)
    t = np.empty((nx, ny, nz), np.uint8)
    f = np.empty((nx, ny, nz, 3), np.float32)
    m = np.empty((nx, ny, nz), np.uint8)
    isl = np.zeros(3)
    N.check(L.lqt_geom_ventricle(C.byref(sp), _p(t), _p(f), _p(m), _p(isl)), "lqt_geom_ventricle")
    return Ventricle(t, f, m, isl, sp)


def mirror_map(types: np.ndarray, gpu: bool = False):
    """(tissue_of, bnd_dst, bnd_src) of a grid: built on the host
    (lqt_geom_mirror_map) or on the GPU as lqt_sim_create builds them
    (lqt_geom_mirror_map_gpu); the two are bit-identical."""
    L = _bind()
    g = np.ascontiguousarray(types, dtype=np.uint8)
    shp = g.shape + (1,) * (3 - g.ndim)
    tissue_of = np.zeros(g.size, np.int32)
    n = C.c_int64()
    if gpu:
        call = lambda *a: L.lqt_geom_mirror_map_gpu(*a, None)  # noqa: E731
    else:
        call = L.lqt_geom_mirror_map
    N.check(call(*shp, _p(g), None, None, None, C.byref(n)), "lqt_geom_mirror_map")
    dst = np.zeros(n.value, np.int64)
    src = np.zeros(n.value, np.int64)
    N.check(call(*shp, _p(g), _p(tissue_of), _p(dst), _p(src), C.byref(n)), "lqt_geom_mirror_map")
    return tissue_of, dst, src


# ---- the reference drivers' input files -------------------------------------
class GeomFileSpec(C.Structure):
    _fields_ = [("dim", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("case_edits", C.c_int32), ("reserved", C.c_int32)]


@dataclass
class LoadedGeometry:
    types: np.ndarray      # cell types per grid voxel (LQT_EMPTY off tissue)
    code: np.ndarray       # the file's code after the case edits (0 off tissue)
    fibre: np.ndarray      # fibre vector per voxel
    s2_mask: np.ndarray
    ntissue: int


def load_geometry(path: str, shape, case_edits: bool = True, fibre: bool = True) -> LoadedGeometry:
    """A geometry text file of the reference (3D: "x y z fx fy fz code",
    GPU3D.cu:1276-1468; 2D: "x y fx fy code", new_11.cu:1296-1478) on a grid
    of `shape` (nx, ny, nz) or (nx, ny)."""
    L = N.lib()
    L.lqt_io_read_geometry.argtypes = [C.c_char_p, C.POINTER(GeomFileSpec), C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.POINTER(C.c_int64)]
    dim = len(shape)
    nx, ny = shape[0], shape[1]
    nz = shape[2] if dim == 3 else 1
    sp = GeomFileSpec(dim, nx, ny, nz, int(case_edits), 0)
    g = (nx, ny, nz) if dim == 3 else (nx, ny)
    types = np.empty(g, np.uint8)
    code = np.empty(g, np.uint8)
    fib = np.empty(g + (3,), np.float32) if fibre else None
    s2 = np.empty(g, np.uint8)
    n = C.c_int64()
    N.check(L.lqt_io_read_geometry(os.fsencode(path), C.byref(sp), _p(types), _p(code), _p(fib), _p(s2), C.byref(n)),
            "lqt_io_read_geometry")
    return LoadedGeometry(types, code, fib, s2, int(n.value))


def load_stimulation(path: str, types: np.ndarray, layer: int = -1):
    """Stimulation profile "x y z a b c onset tag" (GPU3D.cu:1694-1712;
    layer >= 0 keeps one z layer for a 2D grid, new_11.cu:1723-1741).
    Returns (s1_mask, onset ms) on the grid of `types`."""
    L = N.lib()
    L.lqt_io_read_stimulation.argtypes = [C.c_char_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p,
                                          C.c_void_p, C.c_void_p, C.POINTER(C.c_int64)]
    t = np.ascontiguousarray(types, np.uint8)
    shp = t.shape + (1,) * (3 - t.ndim)
    mask = np.empty(t.shape, np.uint8)
    onset = np.empty(t.shape, np.float32)
    n = C.c_int64()
    N.check(L.lqt_io_read_stimulation(os.fsencode(path), shp[0], shp[1], shp[2], layer, _p(t), _p(mask), _p(onset),
                                      C.byref(n)), "lqt_io_read_stimulation")
    return mask, onset
