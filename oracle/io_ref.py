"""Restatement of the reference drivers' output loops (test infrastructure:
the checker for the C ABI writers, never the thing measured or shipped).

* vtk_text: GPU3D.cu:123-163 / new_11.cu:142-180 writeData() -- header with
  DIMENSIONS X/s Y/s Z/s (integer division), then for z, y, x in steps of s
  (x innermost) the value of the voxel as a C++ stream prints a double (%g) or
  "-100" where the grid has no tissue, each followed by a space; a newline
  after every x row and another after every z plane.
* dat_text: OneD.cc:402-415, SingleCell.cc:113-139, OneD_VW.cc -- "%4.10f\\t"
  per value and a newline per row.
"""
from __future__ import annotations

import numpy as np


def vtk_text(v_grid, tissue, stride):
    """v_grid, tissue: arrays of shape (X, Y, Z) (or (X, Y) for 2D)."""
    v = np.asarray(v_grid, np.float64)
    t = np.asarray(tissue, bool)
    if v.ndim == 2:
        v, t = v[:, :, None], t[:, :, None]
    X, Y, Z = v.shape
    out = ["# vtk DataFile Version 3.0\n", "vtk output\n", "ASCII\n", "DATASET STRUCTURED_POINTS\n",
           f"DIMENSIONS {X // stride} {Y // stride} {Z // stride}\n", "SPACING 1 1 1\n", "ORIGIN 0 0 0\n",
           f"POINT_DATA {(X // stride) * (Y // stride) * (Z // stride)}\n", "SCALARS ImageFile float 1\n",
           "LOOKUP_TABLE default\n"]
    for z in range(0, Z, stride):
        for y in range(0, Y, stride):
            row = []
            for x in range(0, X, stride):
                row.append(("%g " % v[x, y, z]) if t[x, y, z] else "-100 ")
            out.append("".join(row) + "\n")
        out.append("\n")
    return "".join(out)


def dat_text(rows):
    rows = np.atleast_2d(np.asarray(rows, np.float64))
    return "".join("".join("%4.10f\t" % x for x in r) + "\n" for r in rows)


# ---- input files -------------------------------------------------------------
EPI_CODES = (7, 8, 9, 10, 17, 18, 19, 20)       # GPU3D.cu:655 and the other type tests
M_CODES = (4, 5, 6, 14, 15, 16)
LQT_EPI, LQT_ENDO, LQT_MCELL, LQT_EMPTY = 2, 3, 4, 255


def read_geometry_points(path, shape, case_edits=True):
    """The same rules, as {grid index tuple: (type, code, s2)} for sparse checks."""
    out = {}
    dim = len(shape)
    for line in open(path):
        f = line.split()
        if not f:
            continue
        if dim == 3:
            x, y, z, fy, code = int(f[0]), int(f[1]), int(f[2]), float(f[4]), int(f[6])
        else:
            x, y, z, fy, code = int(f[0]), int(f[1]), 0, float(f[3]), int(f[4])
        s2 = False
        if case_edits:
            if dim == 3:
                s2 = 300 <= x < 687 and 120 <= y < 486 and 420 <= z < 534
                if 4 <= code <= 6:
                    code = 2 if fy <= 4 else 7
                dist = ((x - 597) ** 2 + (y - 336) ** 2 + (z - 336) ** 2) ** 0.5
                if 14 <= code <= 16 and not dist < 75:
                    code = 12 if code <= 14 else 17
            else:
                s2 = 300 <= x < 400 and 200 <= y < 350 and 11 <= code <= 13
                if 3 <= code <= 6:
                    code = 2 if code <= 4 else 7
                if 13 <= code <= 16 and not (550 <= x < 689 and 150 <= y < 487):
                    code = 12 if code <= 14 else 17
        t = LQT_EPI if code in EPI_CODES else (LQT_MCELL if code in M_CODES else LQT_ENDO)
        out[(x, y, z) if dim == 3 else (x, y)] = (t, code, int(s2))
    return out


def read_geometry(path, shape, case_edits=True, fibre=True):
    """GPU3D.cu:1276-1468 (3D) / new_11.cu:1296-1478 (2D), line by line."""
    dim = len(shape)
    g = tuple(shape)
    types = np.full(g, LQT_EMPTY, np.uint8)
    code_g = np.zeros(g, np.uint8)
    fib = np.zeros(g + (3,), np.float32) if fibre else None
    s2m = np.zeros(g, np.uint8)
    n = 0
    for line in open(path):
        f = line.split()
        if not f:
            continue
        if dim == 3:
            x, y, z = int(f[0]), int(f[1]), int(f[2])
            fx, fy, fz = float(f[3]), float(f[4]), float(f[5])
            code = int(f[6])
        else:
            x, y, z = int(f[0]), int(f[1]), 0
            fx, fy, fz = float(f[2]), float(f[3]), 0.0
            code = int(f[4])
        s2 = False
        if case_edits:
            if dim == 3:
                s2 = 300 <= x < 687 and 120 <= y < 486 and 420 <= z < 534
                if 4 <= code <= 6:
                    code = 2 if fy <= 4 else 7
                dist = ((x - 597) ** 2 + (y - 336) ** 2 + (z - 336) ** 2) ** 0.5
                if 14 <= code <= 16 and not dist < 75:
                    code = 12 if code <= 14 else 17
            else:
                s2 = 300 <= x < 400 and 200 <= y < 350 and 11 <= code <= 13
                if 3 <= code <= 6:
                    code = 2 if code <= 4 else 7
                if 13 <= code <= 16 and not (550 <= x < 689 and 150 <= y < 487):
                    code = 12 if code <= 14 else 17
        idx = (x, y, z) if dim == 3 else (x, y)
        types[idx] = LQT_EPI if code in EPI_CODES else (LQT_MCELL if code in M_CODES else LQT_ENDO)
        code_g[idx] = code
        if fib is not None:
            fib[idx] = (fx, fy, fz)
        s2m[idx] = s2
        n += 1
    return types, code_g, fib, s2m, n


def read_stimulation(path, types, layer=-1):
    """GPU3D.cu:1694-1712 / new_11.cu:1723-1741."""
    mask = np.zeros(types.shape, np.uint8)
    onset = np.zeros(types.shape, np.float32)
    for line in open(path):
        f = line.split()
        if not f:
            continue
        x, y, z = int(f[0]), int(f[1]), int(f[2])
        on = np.float32(float(f[6]))
        if layer >= 0:
            if z != layer:
                continue
            idx = (x, y)
        else:
            idx = (x, y, z)
        if any(i < 0 or i >= s for i, s in zip(idx, types.shape)):
            continue
        if types[idx] == LQT_EMPTY:
            continue
        mask[idx] = 1
        onset[idx] = on
    return mask, onset
