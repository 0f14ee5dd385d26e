"""lqt_ecg_grid_noalloc: the pseudo-ECG entry point that allocates nothing.

It exists for callers that cannot call cudaMalloc themselves or let a library
do it: a host framework that owns all device memory and hands out fixed
buffers, or a stepping loop that must avoid the device-wide synchronisation of
cudaMalloc/cudaFree.  Such a caller passes its own V grid, tissue index and
output buffer; the library uses a fixed device array for its scratch.  This
test gives it caller-owned device buffers (allocated here, by the caller, with
torch) and checks it against the ECG the simulation computes with its own
buffers, on two calls in a row.  It sits in a file that pytest collects last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_ecg_matches_simulation_ecg_twice():
    import torch

    import lqt1_gb300 as lq
    L = lq.lib()
    L.lqt_ecg_grid_noalloc.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_void_p,
                                       C.c_int64, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]
    L.lqt_ecg_grid_noalloc.restype = C.c_int

    sh = lq.geometry.sheet(48, 40, s1_cols=3)
    electrodes = np.array([[-3.0, 4.0, 2.0], [9.0, 5.0, -1.5], [3.0, 12.0, 0.5]])
    sim = lq.Sim(sh.types, 0.15, precision=lq.MIXED, model="default")
    sim.set_protocol(bcl=1000.0, s1_mask=sh.s1_mask, s1_duration=2.0)
    sim.set_electrodes(electrodes, every=50)
    sim.step(400)                                   # wave in flight; 8 samples
    phi_sim, _ = sim.ecg()
    want = phi_sim[-1]
    assert np.abs(want).max() > 0

    # caller-owned device inputs: dense V grid with mirror ghosts, tissue index
    v = sim.get_v()
    tidx = sim.tissue_index()
    dst, src = sim.boundary()
    grid = np.zeros(sh.types.size, np.float32)
    grid[tidx] = v
    grid[dst] = grid[src]
    v_dev = torch.from_numpy(grid).cuda()
    idx_dev = torch.from_numpy(tidx.astype(np.int32)).cuda()
    out_dev = torch.zeros(len(electrodes), dtype=torch.float64, device="cuda")
    el = np.ascontiguousarray(electrodes)
    nx, ny = sh.types.shape
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        out_dev.fill_(np.nan)
        rc = L.lqt_ecg_grid_noalloc(v_dev.data_ptr(), nx, ny, 1, 0.15, idx_dev.data_ptr(), len(tidx),
                                    el.ctypes.data, len(electrodes), out_dev.data_ptr(), stream)
        assert rc == 0, L.lqt_last_error()
        torch.cuda.synchronize()
        got = out_dev.cpu().numpy()
        np.testing.assert_allclose(got, want, rtol=1e-9, atol=1e-12 * np.abs(want).max())

    # sizes beyond the limit are refused with a message, nothing launched
    el9 = np.zeros((9, 3))
    rc = L.lqt_ecg_grid_noalloc(v_dev.data_ptr(), nx, ny, 1, 0.15, idx_dev.data_ptr(), len(tidx), el9.ctypes.data,
                                9, out_dev.data_ptr(), stream)
    assert rc == 1 and b"nel must be 1..8" in L.lqt_last_error()
