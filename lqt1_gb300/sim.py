"""Tissue simulations on the GPU (lqt_sim_*): 1D strands, 2D sheets, 3D volumes.

`Sim` is the host-side handle of the drivers the reference writes as single
`main()` programs (OneD.cc, new_11.cu, GPU3D.cu): geometry, stimulus protocol,
stepping, V read-back, pseudo-ECG, activation / APD90 detectors, blow-up
check and checkpoints.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _native as N


def _p(a):
    return None if a is None else a.ctypes.data


class Sim:
    def __init__(self, types: np.ndarray, dx: float, *, fibre: np.ndarray | None = None, d_fibre: float = 0.154,
                 d_trans: float = 0.0385, coeff_1d: np.ndarray | None = None, precision: int = N.MIXED,
                 model: N.Model | str = "default", dt: float = 0.02, v0: float = -87.5, detect: bool = True,
                 act_threshold: float = -30.0, vmin_ok: float = -200.0, vmax_ok: float = 200.0,
                 stream: int | None = None):
        t = np.ascontiguousarray(types, dtype=np.uint8)
        self.shape = t.shape
        dims = t.shape + (1,) * (3 - t.ndim)
        self.types = t
        self.dx = dx
        f = None if fibre is None else np.ascontiguousarray(fibre, dtype=np.float32)
        c1 = None if coeff_1d is None else np.ascontiguousarray(coeff_1d, dtype=np.float64)
        self._keep = (t, f, c1)
        geom = N.Geometry(dims[0], dims[1], dims[2], dx, _p(t), _p(f), d_fibre, d_trans, _p(c1))
        m = N.model(model) if isinstance(model, str) else model
        self.model = m
        p = N.SimParams(dt, v0, precision, int(detect), m, act_threshold, vmin_ok, vmax_ok, C.c_void_p(stream or 0))
        h = C.c_void_p()
        N.check(N.lib().lqt_sim_create(C.byref(p), C.byref(geom), C.byref(h)), "lqt_sim_create")
        self._h = h
        self.n = int(N.lib().lqt_sim_num_tissue(h))
        self.dt = dt
        self.precision = precision
        self.nel = 0

    def close(self):
        if getattr(self, "_h", None):
            N.lib().lqt_sim_destroy(self._h)
            self._h = None

    __del__ = close

    # ---- protocol ----------------------------------------------------------
    def set_protocol(self, *, bcl: float, s1_mask: np.ndarray, s1_start: float = 0.0, s1_duration: float = 2.0,
                     s1_strength: float = -52.0, s1_beats: int = 0, s1_onset: np.ndarray | None = None,
                     s2_time: float = -1.0, s2_duration: float = 0.0, s2_strength: float = 0.0,
                     s2_mask: np.ndarray | None = None):
        m1 = np.ascontiguousarray(s1_mask, dtype=np.uint8).reshape(-1)
        m2 = None if s2_mask is None else np.ascontiguousarray(s2_mask, dtype=np.uint8).reshape(-1)
        on = None if s1_onset is None else np.ascontiguousarray(s1_onset, dtype=np.float32).reshape(-1)
        q = N.Protocol(bcl, s1_start, s1_duration, s1_strength, s1_beats, 0, _p(m1), _p(on), s2_time, s2_duration,
                       s2_strength, _p(m2))
        N.check(N.lib().lqt_sim_set_protocol(self._h, C.byref(q)), "lqt_sim_set_protocol")

    # ---- stepping ------------------------------------------------------------
    def step(self, nsteps: int = 1):
        N.check(N.lib().lqt_sim_step(self._h, int(nsteps)), "lqt_sim_step")

    def step_async(self, nsteps: int = 1):
        """Enqueue nsteps steps without waiting for them (see lqt_sim_step_async)."""
        N.check(N.lib().lqt_sim_step_async(self._h, int(nsteps)), "lqt_sim_step_async")

    def sync(self):
        """Wait for every enqueued step."""
        N.check(N.lib().lqt_sim_sync(self._h), "lqt_sim_sync")

    @property
    def time(self) -> float:
        return float(N.lib().lqt_sim_time(self._h))

    # ---- read-back -------------------------------------------------------------
    def get_v(self, as_double: bool = False) -> np.ndarray:
        out = np.zeros(self.n, np.float64 if as_double else np.float32)
        N.check(N.lib().lqt_sim_get_v(self._h, _p(out), int(as_double)), "lqt_sim_get_v")
        return out

    def get_v_into(self, out: np.ndarray):
        """V into a caller buffer (float32 or float64, length n)."""
        N.check(N.lib().lqt_sim_get_v(self._h, _p(out), int(out.dtype == np.float64)), "lqt_sim_get_v")

    def get_v_async(self, out: np.ndarray) -> int:
        """Start copying V into `out` (pinned for overlap).  Returns the
        copy's number (0, 1, ... over this simulation's life): `out` is
        complete after wait_v(number) or wait_v()."""
        L = N.lib()
        L.lqt_sim_get_v_async.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        N.check(L.lqt_sim_get_v_async(self._h, _p(out), int(out.dtype == np.float64)), "lqt_sim_get_v_async")
        self._v_issued = getattr(self, "_v_issued", 0) + 1
        return self._v_issued - 1

    def wait_v(self, upto: int | None = None):
        """Wait for every read-back copy in flight, or (upto) for copies
        0..upto only."""
        L = N.lib()
        if upto is None:
            L.lqt_sim_wait_v.argtypes = [C.c_void_p]
            N.check(L.lqt_sim_wait_v(self._h), "lqt_sim_wait_v")
        else:
            L.lqt_sim_wait_v_upto.argtypes = [C.c_void_p, C.c_int64]
            N.check(L.lqt_sim_wait_v_upto(self._h, int(upto)), "lqt_sim_wait_v_upto")

    def tissue_index(self) -> np.ndarray:
        out = np.zeros(self.n, np.int64)
        N.check(N.lib().lqt_sim_tissue_index(self._h, _p(out)), "lqt_sim_tissue_index")
        return out

    def v_grid(self, fill=np.nan) -> np.ndarray:
        g = np.full(self.types.size, fill, np.float32)
        g[self.tissue_index()] = self.get_v()
        return g.reshape(self.shape)

    def get_state(self, out: np.ndarray | None = None) -> np.ndarray:
        s = np.zeros((self.n, N.NSTATE)) if out is None else out
        assert s.dtype == np.float64 and s.flags.c_contiguous and s.size == self.n * N.NSTATE
        N.check(N.lib().lqt_sim_get_state(self._h, _p(s)), "lqt_sim_get_state")
        return s

    def set_state(self, s: np.ndarray):
        s = np.ascontiguousarray(s, dtype=np.float64)
        N.check(N.lib().lqt_sim_set_state(self._h, _p(s)), "lqt_sim_set_state")

    def tune(self, variant: int = -1):
        """Force an occupancy variant of the step kernel (>= 0) or autotune now (-1).
        Returns (chosen variant, ms per candidate)."""
        L = N.lib()
        L.lqt_sim_tune.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.c_void_p]
        ch = C.c_int32()
        ms = np.zeros(4, np.float32)
        N.check(L.lqt_sim_tune(self._h, int(variant), C.byref(ch), _p(ms)), "lqt_sim_tune")
        return ch.value, ms

    def substep_variant(self, variant: int = -1, timings: bool = False):
        """Force the V-only substep's kernel variant (5, 6, 8 direct; 105, 106,
        108 staged by bulk copies; 203, 204 with the V halo staged too; 304,
        305, 306 rows streamed by a producer warp) or,
        with -1, report the current one; with timings, also the last
        autotune's ms per variant (same order)."""
        L = N.lib()
        L.lqt_sim_substep_variant.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.c_void_p]
        ch = C.c_int32()
        ms = np.zeros(11, np.float32)
        N.check(L.lqt_sim_substep_variant(self._h, int(variant), C.byref(ch), _p(ms)), "lqt_sim_substep_variant")
        return (ch.value, ms) if timings else ch.value

    def profile(self, nsteps: int = 20):
        """Mean device ms per launch of the fused step kernel, of the ghost
        kernel and (with a surrogate attached) of the surrogate macro-step
        kernel, 0 when none ran (CUDA events on the simulation's stream)."""
        L = N.lib()
        L.lqt_sim_profile.argtypes = [C.c_void_p, C.c_int64] + [C.POINTER(C.c_double)] * 3
        a, b, c = C.c_double(), C.c_double(), C.c_double()
        N.check(L.lqt_sim_profile(self._h, int(nsteps), C.byref(a), C.byref(b), C.byref(c)), "lqt_sim_profile")
        return a.value, b.value, c.value

    # ---- output files ----------------------------------------------------------------
    def sample_v(self, stride: int = 3) -> np.ndarray:
        """V on the VTK lattice (every `stride`-th voxel per axis, z outermost,
        x innermost, -100 off tissue), sampled on the device."""
        L = N.lib()
        L.lqt_sim_sample_v.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]
        n = C.c_int64()
        N.check(L.lqt_sim_sample_v(self._h, stride, None, 0, C.byref(n)), "lqt_sim_sample_v")
        out = np.zeros(n.value)
        N.check(L.lqt_sim_sample_v(self._h, stride, _p(out), n.value, C.byref(n)), "lqt_sim_sample_v")
        return out

    def vtk_writer(self, stride: int = 3, nbuf: int = 2) -> "VtkWriter":
        return VtkWriter(self, stride, nbuf)

    # ---- learned surrogate ---------------------------------------------------------
    def set_surrogate(self, mlp=None, *, dvdt_max: float = 1.5, kappa: float = 1.5, vstep_max: float = 0.4,
                      use_net: bool = True, nsub: int | None = None, foot_dvdt: float = 0.1, foot_v: float = -40.0):
        """Attach a trained surrogate network (lqt1_gb300.surrogate.Mlp) or
        detach (None).  Mixed form only; see lqt_sim_set_surrogate.  The macro
        step is the network's own length (mlp.nsub plain steps) unless nsub
        overrides it; foot_dvdt > 0 keeps voxels below foot_v whose V rises
        faster than foot_dvdt (mV/ms) on the plain step (the foot of a wave;
        0 = off)."""
        L = N.lib()
        L.lqt_sim_set_surrogate.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        if mlp is None:
            N.check(L.lqt_sim_set_surrogate(self._h, None, None), "lqt_sim_set_surrogate")
            self._sur = None
            return
        cfg = N.SurConfig(dvdt_max, kappa, vstep_max, int(bool(use_net)), int(nsub or getattr(mlp, "nsub", 5)),
                          float(foot_dvdt), float(foot_v))
        N.check(L.lqt_sim_set_surrogate(self._h, mlp._h, C.byref(cfg)), "lqt_sim_set_surrogate")
        self._sur = mlp     # keep the network alive while attached

    def surrogate_stats(self, reset: bool = False):
        """Macro steps launched, voxel offers, voxels accepted, wait timeouts."""
        L = N.lib()
        L.lqt_sim_surrogate_stats.argtypes = [C.c_void_p] + [C.POINTER(C.c_int64)] * 3 + [C.POINTER(C.c_int32),
                                                                                             C.c_int32]
        m, o, a = C.c_int64(), C.c_int64(), C.c_int64()
        t = C.c_int32()
        N.check(L.lqt_sim_surrogate_stats(self._h, C.byref(m), C.byref(o), C.byref(a), C.byref(t), int(reset)),
                "lqt_sim_surrogate_stats")
        return dict(macro_steps=m.value, offered=o.value, accepted=a.value, wait_timeouts=t.value)

    def set_wait_test(self, skip_first_copy: bool, wait_limit: int = 0):
        """Failure-path test (lqt_sim_set_wait_test): make the staged substep's
        first tile wait of every CTA run out after wait_limit polls."""
        L = N.lib()
        L.lqt_sim_set_wait_test.argtypes = [C.c_void_p, C.c_int32, C.c_uint32]
        N.check(L.lqt_sim_set_wait_test(self._h, int(bool(skip_first_copy)), int(wait_limit)),
                "lqt_sim_set_wait_test")

    def surrogate_rejections(self):
        """Offered voxels that failed each residual check since the last
        reset: network bound, gate range, concentration, ionic V step."""
        L = N.lib()
        L.lqt_sim_surrogate_rejections.argtypes = [C.c_void_p, C.c_void_p]
        c = np.zeros(4, np.int64)
        N.check(L.lqt_sim_surrogate_rejections(self._h, _p(c)), "lqt_sim_surrogate_rejections")
        return dict(zip(("network_bound", "gate_range", "concentration", "v_step"), (int(x) for x in c)))

    def boundary(self):
        L = N.lib()
        L.lqt_sim_boundary.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_int64)]
        n = C.c_int64()
        N.check(L.lqt_sim_boundary(self._h, None, None, C.byref(n)), "lqt_sim_boundary")
        d = np.zeros(n.value, np.int64)
        s = np.zeros(n.value, np.int64)
        N.check(L.lqt_sim_boundary(self._h, _p(d), _p(s), C.byref(n)), "lqt_sim_boundary")
        return d, s

    # ---- pseudo-ECG --------------------------------------------------------------
    def set_electrodes(self, xyz, every: int = 50):
        xyz = np.ascontiguousarray(np.asarray(xyz, np.float64).reshape(-1, 3))
        self.nel = len(xyz)
        N.check(N.lib().lqt_sim_set_electrodes(self._h, len(xyz), _p(xyz), every), "lqt_sim_set_electrodes")

    def ecg(self):
        n = C.c_int64()
        N.check(N.lib().lqt_sim_get_ecg(self._h, 0, None, None, C.byref(n)), "lqt_sim_get_ecg")
        phi = np.zeros((n.value, self.nel))
        t = np.zeros(n.value)
        N.check(N.lib().lqt_sim_get_ecg(self._h, n.value, _p(phi), _p(t), C.byref(n)), "lqt_sim_get_ecg")
        return phi, t

    # ---- detectors / checks -----------------------------------------------------------
    def detect(self):
        t_act = np.zeros(self.n, np.float32)
        apd = np.zeros(self.n, np.float32)
        ead = np.zeros(self.n, np.uint8)
        N.check(N.lib().lqt_sim_get_detect(self._h, _p(t_act), _p(apd), _p(ead)), "lqt_sim_get_detect")
        return dict(t_act=t_act, apd90=apd, ead=ead)

    def check(self) -> int:
        n = C.c_int64()
        rc = N.lib().lqt_sim_check(self._h, C.byref(n))
        if rc not in (N.OK, N.ERR_NUMERIC):
            N.check(rc, "lqt_sim_check")
        return int(n.value)

    def checkpoint(self, path: str):
        N.check(N.lib().lqt_sim_checkpoint(self._h, path.encode()), "lqt_sim_checkpoint")

    def restore(self, path: str):
        N.check(N.lib().lqt_sim_restore(self._h, path.encode()), "lqt_sim_restore")


class VtkWriter:
    """Asynchronous VTK snapshots of a Sim (lqt_vtk_writer_*): submit(path)
    samples V on the device and returns; a host thread writes the file."""

    def __init__(self, sim: Sim, stride: int = 3, nbuf: int = 2):
        L = N.lib()
        L.lqt_vtk_writer_create.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]
        L.lqt_vtk_writer_submit.argtypes = [C.c_void_p, C.c_char_p]
        L.lqt_vtk_writer_flush.argtypes = [C.c_void_p]
        L.lqt_vtk_writer_destroy.argtypes = [C.c_void_p]
        L.lqt_vtk_writer_destroy.restype = None
        h = C.c_void_p()
        N.check(L.lqt_vtk_writer_create(sim._h, stride, nbuf, C.byref(h)), "lqt_vtk_writer_create")
        self._h, self._sim, self.L = h, sim, L

    def submit(self, path: str):
        N.check(self.L.lqt_vtk_writer_submit(self._h, os.fsencode(path)), "lqt_vtk_writer_submit")

    def flush(self):
        N.check(self.L.lqt_vtk_writer_flush(self._h), "lqt_vtk_writer_flush")

    def close(self):
        if getattr(self, "_h", None):
            self.L.lqt_vtk_writer_destroy(self._h)
            self._h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.flush()
        self.close()
