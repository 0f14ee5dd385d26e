"""ctypes bindings of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

The oracle (oracle/lqt_oracle.c) restates the reference's FP64 TPORd path
(SingleCell/TPORd.cc:379-1021, OneD.cc:100-436, SingleCell.cc:95-232,
GPU3D.cu:1487-1680, new_11.cu:352-417, PlotScript/plot1DECG_compare.py:89-105).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liblqt_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")

NSTATE = 40
LVEPI, LVENDO, EPI, ENDO, MCELL, EMPTY = 0, 1, 2, 3, 4, 255


class Model(C.Structure):
    """Mirror of `lqt_model` in include/lqt.h."""

    _fields_ = [
        ("dss_shift", C.c_double),
        ("fss_shift", C.c_double),
        ("pca_scale", C.c_double),
        ("gks_scale", C.c_double),
        ("gks_iso_scale", C.c_double),
        ("suprep_dose", C.c_double),
        ("reserved", C.c_double * 2),
    ]


# The reference's builds (SingleCell/TPORd.cc:30-36, GPU3D.cu:18-22, new_11.cu:18-21).
PRESETS = {
    "baseline": dict(dss_shift=0.0, fss_shift=0.0, pca_scale=1.0, gks_scale=1.0, gks_iso_scale=1.0, suprep_dose=0.0),
    "default": dict(dss_shift=12.0, fss_shift=8.0, pca_scale=1.6, gks_scale=1.0, gks_iso_scale=3.2, suprep_dose=0.0),
    "con": dict(dss_shift=0.0, fss_shift=0.0, pca_scale=1.0, gks_scale=1.0, gks_iso_scale=1.0, suprep_dose=0.0),
    "lqt1": dict(dss_shift=0.0, fss_shift=0.0, pca_scale=1.0, gks_scale=0.05, gks_iso_scale=1.0, suprep_dose=0.0),
    "lqt1half": dict(dss_shift=0.0, fss_shift=0.0, pca_scale=1.0, gks_scale=0.5, gks_iso_scale=1.0, suprep_dose=0.0),
    "suprep": dict(dss_shift=12.0, fss_shift=8.0, pca_scale=1.6, gks_scale=1.0, gks_iso_scale=3.2, suprep_dose=150.0),
    "gpu3d": dict(dss_shift=12.0, fss_shift=8.0, pca_scale=4.0, gks_scale=0.05, gks_iso_scale=3.2, suprep_dose=100.0),
    "gpu2d": dict(dss_shift=0.0, fss_shift=0.0, pca_scale=1.0, gks_scale=0.05, gks_iso_scale=1.0, suprep_dose=0.0),
}


def model(name_or_dict="default", **over) -> Model:
    d = dict(PRESETS[name_or_dict]) if isinstance(name_or_dict, str) else dict(name_or_dict)
    d.update(over)
    m = Model()
    for k, v in d.items():
        setattr(m, k, float(v))
    return m


class StrandCfg(C.Structure):
    _fields_ = [
        ("n", C.c_int32),
        ("dx", C.c_double),
        ("dt", C.c_double),
        ("bcl", C.c_double),
        ("stim_start", C.c_double),
        ("stim_dur", C.c_double),
        ("stim_strength", C.c_double),
        ("n_stim", C.c_int32),
        ("num_s1", C.c_int32),
        ("stop_time", C.c_double),
        ("act_thr", C.c_double),
    ]


_lib = None


def build(quiet: bool = True) -> str:
    """Compile the oracle with its Makefile (gcc, -O3 -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-f", os.path.join(HERE, "Makefile")], check=True,
                   stdout=subprocess.DEVNULL if quiet else None)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        P = C.c_void_p
        L.orc_initial_state.argtypes = [C.c_double, P]
        L.orc_update.argtypes = [P, C.c_int, C.POINTER(Model), C.c_double, C.c_double, C.c_double, P]
        L.orc_cells_update.argtypes = [C.c_int64, P, P, C.POINTER(Model), C.c_double, P, P, C.c_int64, C.c_int]
        L.orc_cells_currents.argtypes = [C.c_int64, P, P, C.POINTER(Model), C.c_double, P, P, C.c_int64, P]
        L.orc_single_cell_run.argtypes = [C.c_int, C.POINTER(Model), C.c_double, C.c_double, C.c_double,
                                          C.c_double, C.c_double, C.c_double, C.c_double, P, C.c_int64, P,
                                          C.c_int64, P]
        L.orc_single_cell_run.restype = C.c_int64
        L.orc_strand_run.argtypes = [C.POINTER(StrandCfg), P, P, C.POINTER(Model), C.c_double, C.c_int64, P, P,
                                     C.c_int64, C.c_int32, P, P, P, C.c_int]
        L.orc_strand_run.restype = C.c_int64
        L.orc_strand_detect.argtypes = [C.POINTER(StrandCfg), C.c_int32, P, P, C.POINTER(Model), C.c_double,
                                        C.c_int32, P, P, P, P, P]
        L.orc_strand_detect.restype = C.c_int64
        L.orc_vw_trial.argtypes = [C.POINTER(StrandCfg), P, P, C.POINTER(Model), C.c_double, C.c_double, C.c_double,
                                   C.c_double, C.c_int32, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double), P,
                                   C.c_int64]
        L.orc_vw_trial.restype = C.c_int64
        L.orc_ecg_1d.argtypes = [C.c_int32, P, C.c_double, C.c_double]
        L.orc_ecg_1d.restype = C.c_double
        L.orc_build_map.argtypes = [C.c_int32, C.c_int32, C.c_int32, P, P]
        L.orc_build_map.restype = C.c_int64
        L.orc_build_tensor.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_double, P, P, C.c_int64, P,
                                       C.c_double, C.c_double, P, P]
        L.orc_grid_step.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_double, P, P, C.c_int64, P, P, P, P,
                                    C.POINTER(Model), C.c_double, P, P, C.c_int]
        L.orc_ecg_grid.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_double, P, P, C.c_int64, P, P]
        L.orc_ecg_grid.restype = C.c_double
        L.orc_in_window.argtypes = [C.c_double, C.c_double, C.c_double, C.c_double]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def initial_state(v0=-87.5, n=1):
    s = np.zeros((n, NSTATE))
    for i in range(n):
        lib().orc_initial_state(v0, _p(s[i]))
    return s


def cells_update(state, types, m: Model, dt=0.02, ist=None, dvgap=None, nsteps=1, nthreads=0):
    """In-place FP64 updates of n cells (state: [n, 40] float64, C-contiguous)."""
    assert state.dtype == np.float64 and state.flags.c_contiguous
    types = np.ascontiguousarray(types, dtype=np.uint8)
    ist = None if ist is None else np.ascontiguousarray(ist, dtype=np.float64)
    dvgap = None if dvgap is None else np.ascontiguousarray(dvgap, dtype=np.float64)
    lib().orc_cells_update(state.shape[0], _p(state), _p(types), C.byref(m), dt, _p(ist), _p(dvgap),
                           nsteps, nthreads)
    return state


def cells_currents(state, types, m: Model, dt=0.02, ist=None, dvgap=None, nsteps=1):
    """In-place FP64 updates of n cells; returns [n, 6] INa, ICaL, IKr, IKs,
    IK1, |dV/dt| of the last update (the TPORd getters)."""
    assert state.dtype == np.float64 and state.flags.c_contiguous
    types = np.ascontiguousarray(types, dtype=np.uint8)
    ist = None if ist is None else np.ascontiguousarray(ist, dtype=np.float64)
    dvgap = None if dvgap is None else np.ascontiguousarray(dvgap, dtype=np.float64)
    cur = np.zeros((state.shape[0], 6))
    lib().orc_cells_currents(state.shape[0], _p(state), _p(types), C.byref(m), dt, _p(ist), _p(dvgap), nsteps,
                             _p(cur))
    return cur


def single_cell_run(ctype=MCELL, m: Model | None = None, v0=-87.5, dt=0.02, bcl=1000.0, nbeats=100.0,
                    stim_start=50.0, stim_dur=1.0, stim_strength=-53.0, trace_every=0, trace_cap=0):
    """SingleCell.cc driver; returns (stats dict, trace, final state)."""
    m = m or model("default")
    stats = np.zeros(10)
    trace = np.zeros(max(trace_cap, 1))
    fin = np.zeros(NSTATE)
    n = lib().orc_single_cell_run(ctype, C.byref(m), v0, dt, bcl, nbeats, stim_start, stim_dur, stim_strength,
                                  _p(stats), trace_every, _p(trace), trace_cap, _p(fin))
    keys = ["rest", "dvdt_max", "overshoot", "amplitude", "apd20", "apd25", "apd50", "apd75", "apd80", "apd90"]
    return dict(zip(keys, stats.tolist())), trace[:n], fin


def strand_run(types, coeff, m: Model, *, dx=0.15, dt=0.02, bcl=1000.0, stim_start=50.0, stim_dur=1.0,
               stim_strength=-52.0, n_stim=3, num_s1=5, stop_time=None, act_thr=-30.0, v0=-87.5,
               rec_every=10, max_beats=16, nthreads=0):
    """OneD.cc driver; returns dict with rec [nrec, n], rec_t, act [n, max_beats], cv, final state."""
    types = np.ascontiguousarray(types, dtype=np.uint8)
    coeff = np.ascontiguousarray(coeff, dtype=np.float64)
    n = len(types)
    if stop_time is None:
        stop_time = num_s1 * bcl + bcl
    cfg = StrandCfg(n, dx, dt, bcl, stim_start, stim_dur, stim_strength, n_stim, num_s1, stop_time, act_thr)
    nsteps_est = int(stop_time / dt) + 2
    cap = nsteps_est // rec_every + 2 if rec_every > 0 else 0
    rec = np.zeros((max(cap, 1), n))
    rec_t = np.zeros(max(cap, 1))
    act = np.zeros((n, max_beats))
    cv = np.zeros(3)
    fin = np.zeros((n, NSTATE))
    nrec = lib().orc_strand_run(C.byref(cfg), _p(types), _p(coeff), C.byref(m), v0, rec_every, _p(rec),
                                _p(rec_t), cap, max_beats, _p(act), _p(cv), _p(fin), nthreads)
    return dict(rec=rec[:nrec], rec_t=rec_t[:nrec], act=act, cv=cv[0], cv_start=cv[1], cv_end=cv[2], final=fin)


def strand_detect(types, coeff, m: Model, *, dx=0.15, dt=0.02, bcl=1000.0, stim_start=50.0, stim_dur=1.0,
                  stim_strength=-52.0, n_stim=3, s1_beats=0, stop_time=2000.0, act_thr=-30.0, v0=-87.5,
                  max_beats=32):
    """Single cell (n = 1) or strand run with the device AP detector definition."""
    types = np.ascontiguousarray(types, dtype=np.uint8)
    coeff = np.ascontiguousarray(coeff, dtype=np.float64)
    n = len(types)
    cfg = StrandCfg(n, dx, dt, bcl, stim_start, stim_dur, stim_strength, n_stim, 0, stop_time, act_thr)
    t_act = np.zeros((n, max_beats))
    apd = np.zeros((n, max_beats))
    ead = np.zeros(n, np.uint8)
    nact = np.zeros(n, np.int32)
    fin = np.zeros((n, NSTATE))
    lib().orc_strand_detect(C.byref(cfg), s1_beats, _p(types), _p(coeff), C.byref(m), v0, max_beats, _p(t_act),
                            _p(apd), _p(ead), _p(nact), _p(fin))
    return dict(t_act=t_act, apd90=apd, ead=ead, nact=nact, final=fin)


def vw_trial(types, coeff, m: Model, s2_time, *, dx=0.15, dt=0.02, bcl=1000.0, num_s1=5, stim_start=0.0,
             stim_dur=3.0, stim_strength=-52.0, n_stim=3, s2_dur=3.0, s2_strength=-104.0, s2_cell0=10, s2_ncells=3,
             v0=-87.5, record=False):
    """One trial of OneD_VW.cc's S1-S2 search (FP64): (maxEndo, maxEpi[, final-cycle V rows])."""
    types = np.ascontiguousarray(types, dtype=np.uint8)
    coeff = np.ascontiguousarray(coeff, dtype=np.float64)
    n = len(types)
    cfg = StrandCfg(n, dx, dt, bcl, stim_start, stim_dur, stim_strength, n_stim, num_s1, num_s1 * bcl, -30.0)
    me, mp = C.c_double(), C.c_double()
    cap = int(bcl / (50 * dt)) + 2 if record else 0
    rec = np.zeros((max(cap, 1), n))
    nr = lib().orc_vw_trial(C.byref(cfg), _p(types), _p(coeff), C.byref(m), v0, s2_time, s2_dur, s2_strength,
                            s2_cell0, s2_ncells, C.byref(me), C.byref(mp), _p(rec) if record else None, cap)
    if record:
        return me.value, mp.value, rec[:nr]
    return me.value, mp.value


def ecg_1d(v, dx=0.15, x0=35.0):
    v = np.ascontiguousarray(v, dtype=np.float64)
    return lib().orc_ecg_1d(len(v), _p(v), dx, x0)


class Grid:
    """Oracle grid (2D/3D) with the reference's mirror-boundary map."""

    def __init__(self, ctype_grid, dx, fibre=None, d_f=0.154, d_t=0.0385):
        g = np.ascontiguousarray(ctype_grid, dtype=np.uint8)
        if g.ndim == 2:
            g = g[:, :, None]
        self.nx, self.ny, self.nz = g.shape
        self.dx = dx
        self.grid = g
        self.tissue_of = np.zeros(g.size, dtype=np.int32)
        self.n = int(lib().orc_build_map(self.nx, self.ny, self.nz, _p(g), _p(self.tissue_of)))
        self.tissue_cell = np.nonzero(g.reshape(-1) != EMPTY)[0].astype(np.int64)
        self.ctype = g.reshape(-1)[self.tissue_cell].copy()
        fib = None if fibre is None else np.ascontiguousarray(fibre, dtype=np.float32).reshape(-1)
        self.d6 = np.zeros((self.n, 6))
        self.b3 = np.zeros((self.n, 3))
        lib().orc_build_tensor(self.nx, self.ny, self.nz, dx, _p(self.tissue_of), _p(self.tissue_cell), self.n,
                               _p(fib), d_f, d_t, _p(self.d6), _p(self.b3))

    def step(self, state, m: Model, dt=0.02, istim=None, nthreads=0):
        du = np.zeros(self.n)
        istim = None if istim is None else np.ascontiguousarray(istim, dtype=np.float64)
        lib().orc_grid_step(self.nx, self.ny, self.nz, self.dx, _p(self.tissue_of), _p(self.tissue_cell), self.n,
                            _p(self.d6), _p(self.b3), _p(state), _p(self.ctype), C.byref(m), dt, _p(istim),
                            _p(du), nthreads)
        return du

    def ecg(self, state, r0):
        r0 = np.ascontiguousarray(r0, dtype=np.float64)
        return lib().orc_ecg_grid(self.nx, self.ny, self.nz, self.dx, _p(self.tissue_of), _p(self.tissue_cell),
                                  self.n, _p(state), _p(r0))


def in_window(time, bcl, start, dur):
    return bool(lib().orc_in_window(time, bcl, start, dur))


# ---- the reference itself, built here by oracle/build_ref.sh (x86 only) ----

def ref_available(variant="default") -> bool:
    return os.path.exists(os.path.join(REF_DIR, f"libtpord_ref_{variant}.so"))


_ref_libs = {}


def ref_lib(variant="default"):
    if variant not in _ref_libs:
        L = C.CDLL(os.path.join(REF_DIR, f"libtpord_ref_{variant}.so"))
        P = C.c_void_p
        L.lqt_ref_update.argtypes = [C.c_int64, P, P, C.c_double, P, P, C.c_int64, P, C.c_int]
        L.lqt_ref_strands.argtypes = [C.c_int64, C.c_int32, P, C.c_double, C.c_double, C.c_double, C.c_int64,
                                      C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]
        L.lqt_ref_strands.restype = C.c_int64
        L.lqt_ref_currents.argtypes = [C.c_int64, P, P, C.c_double, P, P, C.c_int64, P]
        L.lqt_ref_write_states.argtypes = [C.c_int64, P, C.c_char_p]
        L.lqt_ref_read_states.argtypes = [C.c_int64, P, C.c_char_p]
        _ref_libs[variant] = L
    return _ref_libs[variant]


def ref_update(state, types, variant="default", dt=0.02, ist=None, dvgap=None, nsteps=1, nthreads=0):
    types = np.ascontiguousarray(types, dtype=np.uint8)
    ist = None if ist is None else np.ascontiguousarray(ist, dtype=np.float64)
    dvgap = None if dvgap is None else np.ascontiguousarray(dvgap, dtype=np.float64)
    ref_lib(variant).lqt_ref_update(state.shape[0], _p(state), _p(types), dt, _p(ist), _p(dvgap), nsteps, None,
                                    nthreads)
    return state


def ref_currents(state, types, variant="default", dt=0.02, ist=None, dvgap=None, nsteps=1):
    """The reference's updates and getters ([n, 6]: INa, ICaL, IKr, IKs, IK1, |dV/dt|)."""
    types = np.ascontiguousarray(types, dtype=np.uint8)
    ist = None if ist is None else np.ascontiguousarray(ist, dtype=np.float64)
    dvgap = None if dvgap is None else np.ascontiguousarray(dvgap, dtype=np.float64)
    cur = np.zeros((state.shape[0], 6))
    ref_lib(variant).lqt_ref_currents(state.shape[0], _p(state), _p(types), dt, _p(ist), _p(dvgap), nsteps,
                                      _p(cur))
    return cur


def ref_write_states(state, path, variant="default"):
    """The reference's outputAllStates of each row of state, one file."""
    state = np.ascontiguousarray(state, dtype=np.float64).reshape(-1, NSTATE)
    assert ref_lib(variant).lqt_ref_write_states(state.shape[0], _p(state), path.encode()) == 0


def ref_read_states(n, path, variant="default"):
    """The reference's readinAllStates of n cells from one file."""
    state = np.zeros((n, NSTATE))
    assert ref_lib(variant).lqt_ref_read_states(n, _p(state), path.encode()) == 0
    return state


def random_states(n, seed=0):
    """Physiologically spread random states for known-answer vectors."""
    rng = np.random.default_rng(seed)
    s = initial_state(-87.5, n)
    s[:, 0] = rng.uniform(-95, 50, n)
    s[:, 1:3] *= rng.uniform(0.8, 1.4, (n, 1))
    s[:, 3:5] *= rng.uniform(0.95, 1.02, (n, 1))
    s[:, 5:7] *= rng.uniform(0.5, 20, (n, 2))
    s[:, 7:9] *= rng.uniform(0.5, 1.5, (n, 2))
    s[:, 9:37] = rng.uniform(0, 1, (n, 28))
    s[:, 37:39] = rng.uniform(0, 0.01, (n, 2))
    s[:, 39] = rng.uniform(0, 0.5, n)
    return s
