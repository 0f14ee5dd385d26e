"""Batches of single cells and 1D strands in one persistent launch (lqt_batch_*).

`OneDStrand` reproduces the reference's OneD.cc driver (strand of endo / M /
epi cells, stimulus to the first cells, mirrored-end diffusion, V written
every 10 steps, CV between cells 10 and 90) on the GPU; `Batch` runs many
such instances, each with its own parameters.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _native as N


def _p(a):
    return None if a is None else a.ctypes.data


@dataclass
class InstanceSpec:
    types: np.ndarray                 # per-cell LQT_* types (length = ncells)
    model: int = 0
    bcl: float = 1000.0
    s1_start: float = 50.0
    s1_duration: float = 1.0
    s1_strength: float = -52.0
    s1_beats: int = 0
    n_stim: int = 3
    dx: float = 0.15
    t_stop: float = 6000.0
    record: bool = False
    ecg_x0: float = 35.0
    act_threshold: float = -30.0
    coeff: np.ndarray | None = None   # per-cell D, default 0.154
    currents: bool = False            # with record: ICaL, IKs of the first cell too
    # S2 (OneD_VW.cc): cells [s2_cell0, s2_cell0 + s2_ncells) at t - s2_base in [s2_offset, + s2_duration)
    s2_base: float = 0.0
    s2_offset: float = 0.0
    s2_duration: float = 0.0
    s2_strength: float = 0.0
    s2_cell0: int = 0
    s2_ncells: int = 0
    track_vmax: bool = False          # maximum V of every cell from t - s2_base >= s2_offset


class Batch:
    def __init__(self, instances: list[InstanceSpec], models: list[N.Model], precision: int = N.MIXED,
                 dt: float = 0.02, v0: float = -87.5, max_beats: int = 32, rec_every: int = 10,
                 threads: int = 0, ctas: int = 0, stream: int | None = None):
        self.instances = instances
        ninst = len(instances)
        arr = (N.Instance * ninst)()
        types, coeffs = [], []
        for i, s in enumerate(instances):
            t = np.ascontiguousarray(s.types, dtype=np.uint8)
            types.append(t)
            coeffs.append(np.full(len(t), 0.154) if s.coeff is None else np.asarray(s.coeff, np.float64))
            a = arr[i]
            a.ncells, a.n_stim, a.model = len(t), s.n_stim, s.model
            a.record = (3 if s.currents else 1) if s.record else 0
            a.s2_base, a.s2_offset, a.s2_duration, a.s2_strength = s.s2_base, s.s2_offset, s.s2_duration, s.s2_strength
            a.s2_cell0, a.s2_ncells, a.track_vmax = s.s2_cell0, s.s2_ncells, int(s.track_vmax)
            a.dx, a.bcl, a.s1_start, a.s1_duration, a.s1_strength = s.dx, s.bcl, s.s1_start, s.s1_duration, s.s1_strength
            a.s1_beats, a.t_stop, a.ecg_x0, a.act_threshold = s.s1_beats, s.t_stop, s.ecg_x0, s.act_threshold
        self.types = np.concatenate(types)
        self.coeff = np.ascontiguousarray(np.concatenate(coeffs))
        self.offsets = np.concatenate([[0], np.cumsum([len(t) for t in types])]).astype(np.int64)
        self.max_beats = max_beats
        marr = (N.Model * len(models))(*models)
        p = N.BatchParams(dt, v0, precision, max_beats, rec_every, threads, ctas, C.c_void_p(stream or 0))
        h = C.c_void_p()
        N.check(N.lib().lqt_batch_create(C.byref(p), ninst, C.cast(arr, C.c_void_p), _p(self.types), _p(self.coeff),
                                         len(models), C.cast(marr, C.c_void_p), C.byref(h)), "lqt_batch_create")
        self._h = h
        self.ncells = int(N.lib().lqt_batch_num_cells(h))

    def close(self):
        if getattr(self, "_h", None):
            N.lib().lqt_batch_destroy(self._h)
            self._h = None

    __del__ = close

    def run(self) -> float:
        """Run every instance to its t_stop; returns device milliseconds."""
        N.check(N.lib().lqt_batch_run(self._h), "lqt_batch_run")
        return float(N.lib().lqt_batch_last_run_ms(self._h))

    def config(self):
        """Launch configuration chosen by the autotuner."""
        L = N.lib()
        L.lqt_batch_config.argtypes = [C.c_void_p] + [C.POINTER(C.c_int32)] * 4
        v = [C.c_int32() for _ in range(4)]
        N.check(L.lqt_batch_config(self._h, *[C.byref(x) for x in v]), "lqt_batch_config")
        return dict(threads=v[0].value, min_ctas_per_sm=v[1].value, ctas=v[2].value, nitems=v[3].value)

    def num_bad(self) -> int:
        return int(N.lib().lqt_batch_num_bad(self._h))

    def detect(self):
        n, nb = self.ncells, self.max_beats
        t_act = np.zeros((n, nb), np.float32)
        apd90 = np.zeros((n, nb), np.float32)
        dvdt = np.zeros((n, nb), np.float32)
        ead = np.zeros(n, np.uint8)
        beats = np.zeros(n, np.int32)
        N.check(N.lib().lqt_batch_get_detect(self._h, _p(t_act), _p(apd90), _p(dvdt), _p(ead), _p(beats)),
                "lqt_batch_get_detect")
        return dict(t_act=t_act, apd90=apd90, dvdt_max=dvdt, ead=ead, beats=beats)

    def record(self, i: int):
        nrec = C.c_int64()
        N.check(N.lib().lqt_batch_get_record(self._h, i, None, None, None, 0, C.byref(nrec)), "lqt_batch_get_record")
        m = nrec.value
        n = len(self.instances[i].types)
        v = np.zeros((m, n))
        t = np.zeros(m)
        ecg = np.zeros(m)
        N.check(N.lib().lqt_batch_get_record(self._h, i, _p(v), _p(t), _p(ecg), m, C.byref(nrec)),
                "lqt_batch_get_record")
        out = dict(v=v, t=t, ecg=ecg)
        if self.instances[i].currents:
            ical, iks = np.zeros(m), np.zeros(m)
            N.check(N.lib().lqt_batch_get_record_currents(self._h, i, _p(ical), _p(iks), m, C.byref(nrec)),
                    "lqt_batch_get_record_currents")
            out.update(ical=ical, iks=iks)
        return out

    def vmax(self):
        """Per cell (input order): maximum V of the track_vmax watch."""
        out = np.zeros(self.ncells, np.float32)
        N.check(N.lib().lqt_batch_get_vmax(self._h, _p(out)), "lqt_batch_get_vmax")
        return out

    def get_state(self):
        s = np.zeros((self.ncells, N.NSTATE))
        N.check(N.lib().lqt_batch_get_state(self._h, _p(s)), "lqt_batch_get_state")
        return s

    def set_state(self, s):
        s = np.ascontiguousarray(s, dtype=np.float64)
        N.check(N.lib().lqt_batch_set_state(self._h, _p(s)), "lqt_batch_set_state")


def oned_types(endo=25, mid=35, epi=40):
    """OneD.cc:60-64 and 136-200: endo, then M, then epi cells."""
    return np.array([N.ENDO] * endo + [N.MCELL] * mid + [N.EPI] * epi, np.uint8)


class OneDStrand:
    """The OneD.cc driver on the GPU: returns V every rec_every steps, CV,
    per-cell activation times / APD90 and the pseudo-ECG."""

    def __init__(self, model: N.Model | str = "default", precision: int = N.MIXED, types=None, bcl=1000.0,
                 num_s1=5, stim_duration=1.0, stim_strength=-52.0, stim_start=50.0, dx=0.15, dt=0.02,
                 rec_every=10, ecg_x0=35.0, stop_time=None):
        types = oned_types() if types is None else np.asarray(types, np.uint8)
        stop = num_s1 * bcl + bcl if stop_time is None else stop_time
        m = N.model(model) if isinstance(model, str) else model
        spec = InstanceSpec(types=types, bcl=bcl, s1_start=stim_start, s1_duration=stim_duration,
                            s1_strength=stim_strength, dx=dx, t_stop=stop, record=True, ecg_x0=ecg_x0)
        self.num_s1, self.bcl, self.dx = num_s1, bcl, dx
        self.batch = Batch([spec], [m], precision=precision, dt=dt, rec_every=rec_every,
                           max_beats=int(np.ceil(stop / bcl)) + 1)

    def run(self):
        ms = self.batch.run()
        rec = self.batch.record(0)
        det = self.batch.detect()
        out = dict(rec=rec["v"], rec_t=rec["t"], ecg=rec["ecg"], device_ms=ms, **det)
        # CV on the last S1 cycle from cells 10 and 90 (OneD.cc:419-444)
        n = len(self.batch.types)
        if n > 90:
            ta = det["t_act"]
            lo = self.num_s1 * self.bcl
            s = [x for x in ta[10] if lo <= x < lo + self.bcl]
            e = [x for x in ta[90] if lo <= x < lo + self.bcl]
            out["cv"] = (self.dx * 80) / (e[0] - s[0]) if s and e else float("nan")
            out["cv_start"] = s[0] if s else float("nan")
            out["cv_end"] = e[0] if e else float("nan")
        return out


def sweep(n=4096, seed=2024, beats=20, p_single=0.5, len_range=(50, 400), bcl_range=(400.0, 2000.0),
          stim_duration=2.0, stim_strength=-52.0, record=0):
    """Seeded sweep of uneven instances (the batched-sweep workload).

    Each instance is a single cell (probability p_single, random type) or a
    strand of U{len_range} cells (OneD.cc's 25/35/40 % endo/M/epi split), with
    its own model: IKs mutation fraction f ~ U[0,1] giving GKs x (1 - 0.95 f)
    (f = 1 is the reference's LQT1 factor 0.05, TPORd.cc:706), beta-adrenergic
    ICaL and IKs multipliers ~ U[1,2] (PCa and GKs ISO factors), BCL ~ U(bcl_range),
    `beats` stimulated cycles; stimulus 2 ms x -52 pA/pF at 50 ms.
    Returns (instances, models, params) with params per instance."""
    rng = np.random.default_rng(seed)
    insts, models, params = [], [], []
    for i in range(n):
        single = rng.random() < p_single
        if single:
            types = np.array([rng.choice([N.ENDO, N.MCELL, N.EPI])], np.uint8)
        else:
            L = int(rng.integers(len_range[0], len_range[1] + 1))
            ne, nm = int(round(0.25 * L)), int(round(0.35 * L))
            types = np.array([N.ENDO] * ne + [N.MCELL] * nm + [N.EPI] * (L - ne - nm), np.uint8)
        f = float(rng.random())
        ical = float(rng.uniform(1.0, 2.0))
        iks = float(rng.uniform(1.0, 2.0))
        bcl = float(rng.uniform(*bcl_range))
        m = N.model("baseline", gks_scale=1.0 - 0.95 * f, pca_scale=ical, gks_iso_scale=iks)
        models.append(m)
        insts.append(InstanceSpec(types=types, model=i, bcl=bcl, s1_start=50.0, s1_duration=stim_duration,
                                  s1_strength=stim_strength, s1_beats=beats, n_stim=1 if single else 3, dx=0.15,
                                  t_stop=beats * bcl, record=i < record))
        params.append(dict(single=single, mut=f, ical=ical, iks=iks, bcl=bcl, ncells=len(types)))
    return insts, models, params
