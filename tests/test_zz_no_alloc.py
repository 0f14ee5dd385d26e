"""lqt_ecg_grid_noalloc: the pseudo-ECG entry point that allocates nothing.

It exists for callers that cannot call cudaMalloc themselves or let a library
do it: a host framework that owns all device memory and hands out fixed
buffers, or a stepping loop that must avoid the device-wide synchronisation of
cudaMalloc/cudaFree.  Such a caller passes its own V grid, tissue index and
output buffer; the library uses a fixed device array for its scratch.  These
tests give it caller-owned device buffers (allocated here, by the caller, with
torch) and check it against the ECG the simulation computes with its own
buffers and against the FP64 oracle's sum, on two calls in a row: a 2D sheet,
a 3D shell large enough that each thread of the grid-stride loop takes several
voxels, and a 1D strand (one-sided differences at the ends, no tissue index).
A tissue index on a grid face is refused on the device (NaN in every output,
no read outside the grid), and the next good call is correct again.  The file
sits where pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NOALLOC_ROWS = 2048 * 256     # tissue voxels one pass of the kernel's grid covers


def _lib():
    import lqt1_gb300 as lq
    L = lq.lib()
    L.lqt_ecg_grid_noalloc.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_void_p,
                                       C.c_int64, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]
    L.lqt_ecg_grid_noalloc.restype = C.c_int
    return lq, L


def _call(L, v_dev, dims, dx, idx_dev, ntissue, electrodes, out_dev, stream):
    import torch
    el = np.ascontiguousarray(electrodes, dtype=np.float64)
    out_dev.fill_(12345.0)
    rc = L.lqt_ecg_grid_noalloc(v_dev.data_ptr(), dims[0], dims[1], dims[2], dx,
                                None if idx_dev is None else idx_dev.data_ptr(), ntissue, el.ctypes.data, len(el),
                                out_dev.data_ptr(), stream)
    assert rc == 0, L.lqt_last_error()
    torch.cuda.synchronize()
    return out_dev.cpu().numpy()


def _ghosted_grid(sim):
    """Caller-side dense V grid: tissue V, mirror ghosts filled, zero elsewhere."""
    grid = np.zeros(sim.types.size, np.float32)
    tidx = sim.tissue_index()
    grid[tidx] = sim.get_v()
    dst, src = sim.boundary()
    grid[dst] = grid[src]
    return grid, tidx


def _abs_terms(grid, tidx, dims, dx, r0):
    """Sum of |term| of the ECG sum in FP64 (scale of the rounding error)."""
    nx, ny, nz = dims
    st = np.array([ny * nz, nz, 1])
    c = np.stack([tidx // st[0], (tidx // nz) % ny, tidx % nz], 1).astype(np.float64)
    g = grid.astype(np.float64)
    h = np.stack([0.5 * (g[tidx + s] - g[tidx - s]) if d > 1 else np.zeros(len(tidx)) for s, d in zip(st, dims)], 1)
    r = c * dx - np.asarray(r0)[None, :]
    return float((np.abs((h * r).sum(1)) / np.linalg.norm(r, axis=1) ** 3).sum())


def test_noalloc_ecg_matches_simulation_ecg_twice():
    import torch
    lq, L = _lib()
    sh = lq.geometry.sheet(48, 40, s1_cols=3)
    electrodes = np.array([[-3.0, 4.0, 2.0], [9.0, 5.0, -1.5], [3.0, 12.0, 0.5]])
    sim = lq.Sim(sh.types, 0.15, precision=lq.MIXED, model="default")
    sim.set_protocol(bcl=1000.0, s1_mask=sh.s1_mask, s1_duration=2.0)
    sim.set_electrodes(electrodes, every=50)
    sim.step(400)                                   # wave in flight; 8 samples
    phi_sim, _ = sim.ecg()
    want = phi_sim[-1]
    assert np.abs(want).max() > 0

    grid, tidx = _ghosted_grid(sim)
    v_dev = torch.from_numpy(grid).cuda()
    idx_dev = torch.from_numpy(tidx.astype(np.int32)).cuda()
    out_dev = torch.zeros(len(electrodes), dtype=torch.float64, device="cuda")
    nx, ny = sh.types.shape
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        got = _call(L, v_dev, (nx, ny, 1), 0.15, idx_dev, len(tidx), electrodes, out_dev, stream)
        np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-12 * np.abs(want).max())

    # sizes beyond the limit are refused with a message, nothing launched
    el9 = np.zeros((9, 3))
    rc = L.lqt_ecg_grid_noalloc(v_dev.data_ptr(), nx, ny, 1, 0.15, idx_dev.data_ptr(), len(tidx), el9.ctypes.data,
                                9, out_dev.data_ptr(), stream)
    assert rc == 1 and b"nel must be 1..8" in L.lqt_last_error()


def test_noalloc_ecg_3d_shell_against_simulation_and_oracle(orc):
    """3D shell of 566k tissue voxels (more than one pass of the kernel's grid,
    so each thread sums several voxels): two calls agree with the simulation's
    own ECG and with the FP64 oracle's sum over the same V."""
    import torch
    lq, L = _lib()
    v = lq.geometry.ventricle(nx=116, ny=116, nz=146, a_out=10.5, c_out=25.0, wall=5.0, z_base=27.0,
                              island_radius=2.5, stim_radius=1.5)
    dims = v.types.shape
    cx, cy, zm = v.spec.cx, v.spec.cy, v.spec.z_base - 0.5 * v.spec.c_out
    electrodes = np.array([[cx + 30.0, cy, zm], [cx, cy - 28.0, zm + 3.0], [cx - 5.0, cy + 2.0, -12.0],
                           [cx + 2.0, cy + 31.0, zm - 4.0]])
    sim = lq.Sim(v.types, 0.2, fibre=v.fibre, precision=lq.MIXED, model="default")
    assert sim.n > NOALLOC_ROWS
    sim.set_protocol(bcl=1000.0, s1_mask=v.s1_mask, s1_duration=2.0)
    sim.set_electrodes(electrodes, every=50)
    sim.step(1500)                                  # 30 ms: the wave spreads from the apex
    want_sim = sim.ecg()[0][-1]
    grid, tidx = _ghosted_grid(sim)
    og = orc.Grid(v.types, 0.2)
    np.testing.assert_array_equal(og.tissue_cell, tidx)
    state = np.zeros((og.n, 40))
    state[:, 0] = grid[tidx]
    want_orc = np.array([og.ecg(state, r0) for r0 in electrodes])
    scale = np.array([_abs_terms(grid, tidx, dims, 0.2, r0) for r0 in electrodes])
    assert (np.abs(want_orc) > 1e-3 * scale).all()  # a sum well above its rounding

    v_dev = torch.from_numpy(grid).cuda()
    idx_dev = torch.from_numpy(tidx.astype(np.int32)).cuda()
    out_dev = torch.zeros(len(electrodes), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        got = _call(L, v_dev, dims, 0.2, idx_dev, len(tidx), electrodes, out_dev, stream)
        # FP32 terms summed in FP64: a few FP32 ulps of the sum of |terms|
        np.testing.assert_allclose(got, want_orc, rtol=0, atol=1e-5 * scale.max())
        np.testing.assert_allclose(got, want_sim, rtol=1e-9, atol=1e-12 * np.abs(want_sim).max())


def test_noalloc_ecg_1d_strand_against_oracle(orc):
    """1D strand (no tissue index; one-sided differences at both ends): the
    electrode on the strand's axis 20 mm past its end gives the reference's 1D
    sum (PlotScript/plot1DECG_compare.py:89-105, the oracle's orc_ecg_1d)."""
    import torch
    lq, L = _lib()
    types = lq.batch.oned_types()
    sim = lq.Sim(types, 0.15, precision=lq.MIXED, model="default")
    mask = np.zeros(len(types), np.uint8)
    mask[:3] = 1
    sim.set_protocol(bcl=1000.0, s1_mask=mask, s1_duration=2.0)
    sim.step(600)                                   # 12 ms: the wave is mid-strand
    vh = sim.get_v()
    want = orc.ecg_1d(vh.astype(np.float64), dx=0.15, x0=35.0)
    d = np.diff(vh.astype(np.float64))
    r = np.arange(len(vh)) * 0.15 - 35.0
    scale = float((np.abs(np.concatenate([[d[0]], 0.5 * (d[1:] + d[:-1]), [d[-1]]])) / r ** 2).sum())
    assert abs(want) > 1e-3 * scale
    v_dev = torch.from_numpy(vh).cuda()
    out_dev = torch.zeros(1, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        got = _call(L, v_dev, (len(vh), 1, 1), 0.15, None, len(vh), [[35.0, 0.0, 0.0]], out_dev, stream)
        np.testing.assert_allclose(got[0], want, rtol=0, atol=1e-5 * scale)


def test_noalloc_ecg_refuses_face_voxels_on_the_device():
    """A tissue index on a grid face (its stencil would leave the grid) is
    checked before any V access: every electrode gets NaN, nothing is read
    outside the caller's buffer, and the next call with a good index is
    correct again (the status word is cleared per call)."""
    import torch
    lq, L = _lib()
    sh = lq.geometry.sheet(20, 16, s1_cols=3)
    sim = lq.Sim(sh.types, 0.15, precision=lq.MIXED, model="default")
    sim.set_protocol(bcl=1000.0, s1_mask=sh.s1_mask, s1_duration=2.0)
    electrodes = np.array([[-3.0, 4.0, 2.0], [9.0, 5.0, -1.5]])
    sim.set_electrodes(electrodes, every=50)
    sim.step(100)
    want = sim.ecg()[0][-1]
    grid, tidx = _ghosted_grid(sim)
    nx, ny = sh.types.shape
    v_dev = torch.from_numpy(grid).cuda()
    out_dev = torch.zeros(len(electrodes), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for bad in (0, ny - 1, (nx - 1) * ny + 3, 5 * ny):     # corner, y face, x face, y = 0 face
        idx = tidx.astype(np.int32).copy()
        idx[len(idx) // 2] = bad
        got = _call(L, v_dev, (nx, ny, 1), 0.15, torch.from_numpy(idx).cuda(), len(idx), electrodes, out_dev, stream)
        assert np.isnan(got).all(), (bad, got)
        good = _call(L, v_dev, (nx, ny, 1), 0.15, torch.from_numpy(tidx.astype(np.int32)).cuda(), len(tidx),
                     electrodes, out_dev, stream)
        np.testing.assert_allclose(good, want, rtol=1e-9, atol=1e-12 * np.abs(want).max())
