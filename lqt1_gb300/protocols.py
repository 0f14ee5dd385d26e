"""Protocols of the reference's drivers run as batched launches, and their
output files.

* `vulnerable_window`: the S1-S2 search of OneD_VW.cc (MODE2: S2 timings from
  `start` upward in `step` increments until exactly one strand end depolarises
  above -10 mV), with every candidate timing a separate instance of one
  persistent batched launch instead of one strand run after another.
* `suprep_sweep`: the SUPREP dose series behind PlotScript/plot1DECG_multiple.py
  (OneD.cc strands with LQT1 + ISO1 and SUPREP doses 0..150 fmol), every dose
  an instance of one launch, with the pseudo-ECG at 35 mm on the device.
* `write_oned_dat`, `write_vw_dat`, `write_single_cell_dat`, `write_vtk`: the
  .dat / .vtk layouts of OneD.cc, OneD_VW.cc, SingleCell.cc, GPU3D.cu and
  new_11.cu through the C ABI writers.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _native as N
from .batch import Batch, InstanceSpec, oned_types


def _io():
    L = N.lib()
    L.lqt_io_write_dat.argtypes = [C.c_char_p, C.c_int64, C.c_int32, C.c_void_p, C.c_int32]
    L.lqt_io_write_vtk.argtypes = [C.c_char_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32]
    return L


def write_dat(path: str, rows, append: bool = False):
    """Rows of "%4.10f\\t" values, one line each (the reference's .dat format)."""
    r = np.ascontiguousarray(np.atleast_2d(np.asarray(rows, np.float64)))
    N.check(_io().lqt_io_write_dat(os.fsencode(path), r.shape[0], r.shape[1], r.ctypes.data, int(append)),
            "lqt_io_write_dat")


def write_oned_dat(path: str, rec_t, rec_v):
    """OneD.cc:402-415: time, then V of every cell, every recorded step."""
    rec_v = np.asarray(rec_v, np.float64)
    write_dat(path, np.column_stack([np.asarray(rec_t, np.float64), rec_v]))


def write_single_cell_dat(path: str, t, v, ical, iks):
    """SingleCell.cc:113-139: time, V, ICaL, IKs."""
    write_dat(path, np.column_stack([t, v, ical, iks]))


def write_vw_dat(path: str, rows_v):
    """OneD_VW.cc: V of every cell every 50 steps of the final cycle."""
    write_dat(path, rows_v)


def write_vtk(path: str, samples, shape, stride: int):
    """Legacy-VTK file of lattice samples (Sim.sample_v) of a grid of `shape`."""
    nx, ny = shape[0], shape[1]
    nz = shape[2] if len(shape) > 2 else 1
    s = np.ascontiguousarray(samples, np.float64)
    N.check(_io().lqt_io_write_vtk(os.fsencode(path), s.ctypes.data, nx, ny, nz, stride), "lqt_io_write_vtk")


# ---------------------------------------------------------------------------
def vw_types():
    """OneD_VW.cc:37-41: 25 endo, 35 M, 40 epi cells."""
    return oned_types(25, 35, 40)


def vw_coeff(n=100, d=0.154, dip_cell=63, dip=0.2):
    """OneD_VW.cc:90-104: D = 0.154 except 0.2 x D at cell 63."""
    c = np.full(n, d)
    if 0 <= dip_cell < n:
        c[dip_cell] = dip * d
    return c


def vulnerable_window(s2_times, *, model="default", precision=N.MIXED, types=None, coeff=None, num_s1=5,
                      bcl=1000.0, stim_duration=3.0, stim_strength=-52.0, s2_duration=3.0, s2_strength=-104.0,
                      s2_cell0=10, s2_ncells=3, boundary=10.0, dt=0.02, stream=None):
    """Every S2 timing of `s2_times` (ms after the start of the last S1 cycle)
    as one instance of a single batched launch.  Returns a dict with per
    timing maxEndo, maxEpi (maximum V of the first / last cell from the S2
    time on) and `vulnerable` = (maxEndo + boundary) * (maxEpi + boundary) <= 0,
    the test of OneD_VW.cc:360-420."""
    s2_times = np.asarray(s2_times, np.float64)
    types = vw_types() if types is None else np.asarray(types, np.uint8)
    coeff = vw_coeff(len(types)) if coeff is None else np.asarray(coeff, np.float64)
    m = N.model(model) if isinstance(model, str) else model
    insts = [InstanceSpec(types=types, model=0, bcl=bcl, s1_start=0.0, s1_duration=stim_duration,
                          s1_strength=stim_strength, s1_beats=0, n_stim=3, dx=0.15, t_stop=num_s1 * bcl, coeff=coeff,
                          s2_base=(num_s1 - 1) * bcl, s2_offset=float(t), s2_duration=s2_duration,
                          s2_strength=s2_strength, s2_cell0=s2_cell0, s2_ncells=s2_ncells, track_vmax=True)
             for t in s2_times]
    b = Batch(insts, [m], precision=precision, dt=dt, max_beats=0, stream=stream)
    ms = b.run()
    vmax = b.vmax()
    c0 = b.offsets[:-1]
    n = len(types)
    endo = vmax[c0].astype(np.float64)
    epi = vmax[c0 + n - 1].astype(np.float64)
    vul = (endo + boundary) * (epi + boundary) <= 0
    cells = int(b.ncells)
    b.close()
    return dict(s2=s2_times, max_endo=endo, max_epi=epi, vulnerable=vul, device_ms=ms,
                cell_steps=cells * int(round(num_s1 * bcl / dt)))


def vw_search(start=260.0, step=0.1, batch=1000, max_batches=10, **kw):
    """OneD_VW.cc MODE2: the first S2 timing from `start` upward (in `step`
    increments) at which the S2 wave blocks in one direction only.  Evaluated
    `batch` timings per launch.  Returns (timing or None, the last batch's
    result dict)."""
    for bi in range(max_batches):
        t = start + step * (bi * batch + np.arange(batch))
        r = vulnerable_window(t, **kw)
        hit = np.flatnonzero(r["vulnerable"])
        if hit.size:
            return float(r["s2"][hit[0]]), r
    return None, r


def vw_final_cycle(s2_time, *, model="default", precision=N.MIXED, num_s1=5, bcl=1000.0, dt=0.02, **kw):
    """V of every cell every 50 steps of the last cycle for one S2 timing (the
    rows of OneD_VW.cc's Outputs/Transmural1D_s2@<t>.dat)."""
    types = vw_types()
    coeff = vw_coeff(len(types))
    m = N.model(model) if isinstance(model, str) else model
    spec = InstanceSpec(types=types, model=0, bcl=bcl, s1_start=0.0, s1_duration=kw.get("stim_duration", 3.0),
                        s1_strength=kw.get("stim_strength", -52.0), s1_beats=0, n_stim=3, dx=0.15,
                        t_stop=num_s1 * bcl, coeff=coeff, record=True, s2_base=(num_s1 - 1) * bcl,
                        s2_offset=float(s2_time), s2_duration=kw.get("s2_duration", 3.0),
                        s2_strength=kw.get("s2_strength", -104.0), s2_cell0=10, s2_ncells=3, track_vmax=True)
    b = Batch([spec], [m], precision=precision, dt=dt, rec_every=50, max_beats=0)
    b.run()
    rec = b.record(0)
    b.close()
    sel = np.floor(rec["t"] / bcl) == num_s1 - 1
    return rec["v"][sel]


# ---------------------------------------------------------------------------
def qt_from_ecg(t, ecg, t_stim, bcl, frac=0.05, t_min=100.0):
    """Project definition (the reference only plots the ECGs): QRS onset =
    stimulus time; T peak = largest |ECG - baseline| from t_stim + t_min to
    the end of the cycle, baseline = the sample before the stimulus; T end =
    the first sample after the peak back within frac x |T peak|.  Returns
    (QT ms, T-peak time ms) or (nan, nan)."""
    t = np.asarray(t)
    e = np.asarray(ecg)
    i0 = int(np.searchsorted(t, t_stim)) - 1
    if i0 < 0:
        return float("nan"), float("nan")
    base = e[i0]
    w = (t >= t_stim + t_min) & (t < t_stim + bcl)
    if not w.any():
        return float("nan"), float("nan")
    idx = np.flatnonzero(w)
    d = np.abs(e[idx] - base)
    ip = idx[int(np.argmax(d))]
    amp = abs(e[ip] - base)
    after = np.flatnonzero((np.arange(len(t)) > ip) & w & (np.abs(e - base) < frac * amp))
    if after.size == 0:
        return float("nan"), float(t[ip])
    return float(t[after[0]] - t_stim), float(t[ip])


def suprep_sweep(doses=tuple(range(0, 160, 10)), *, precision=N.MIXED, bcl=1000.0, num_s1=5, stim_start=50.0,
                 stim_duration=1.0, stim_strength=-52.0, rec_every=10, ecg_x0=35.0, dt=0.02, out_dir=None,
                 stream=None):
    """OneD.cc strands with LQT1 + ISO1 and SUPREP at each dose
    (SingleCell/TPORd.cc:709-728), one instance per dose in one launch.  V and
    the pseudo-ECG (x0 = 35 mm, PlotScript/plot1DECG_multiple.py:73-89) every
    rec_every steps.  Returns per dose the ECG, its QT (qt_from_ecg on the last
    complete cycle) and the APD90 of every cell in that cycle.  With out_dir,
    writes VentOneDResults_LQT1_wISO_<dose>.dat files in the OneD.cc layout."""
    types = oned_types()
    stop = num_s1 * bcl + bcl
    models = [N.model("default", gks_scale=0.05, suprep_dose=float(d)) for d in doses]
    insts = [InstanceSpec(types=types, model=i, bcl=bcl, s1_start=stim_start, s1_duration=stim_duration,
                          s1_strength=stim_strength, s1_beats=0, n_stim=3, dx=0.15, t_stop=stop, record=True,
                          ecg_x0=ecg_x0) for i in range(len(doses))]
    b = Batch(insts, models, precision=precision, dt=dt, rec_every=rec_every,
              max_beats=int(np.ceil(stop / bcl)) + 1, stream=stream)
    ms = b.run()
    det = b.detect()
    out = []
    t_last = num_s1 * bcl + stim_start - bcl      # last cycle with a full window before stop
    for i, d in enumerate(doses):
        rec = b.record(i)
        qt, tpk = qt_from_ecg(rec["t"], rec["ecg"], t_last, bcl)
        c0 = b.offsets[i]
        ta = det["t_act"][c0:c0 + len(types)]
        ap = det["apd90"][c0:c0 + len(types)]
        apd_last = np.full(len(types), -1.0)
        for j in range(len(types)):
            k = np.flatnonzero((ta[j] >= t_last) & (ta[j] < t_last + bcl))
            if k.size:
                apd_last[j] = ap[j, k[0]]
        if out_dir:
            write_oned_dat(os.path.join(out_dir, f"VentOneDResults_LQT1_wISO_{int(d)}.dat"), rec["t"], rec["v"])
        out.append(dict(dose=float(d), t=rec["t"], ecg=rec["ecg"], qt=qt, t_peak=tpk, apd90=apd_last))
    b.close()
    return dict(results=out, device_ms=ms)


def main():
    """python -m lqt1_gb300.protocols vw|suprep [--fp64] [--out DIR]: one JSON line."""
    import argparse
    import json
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["vw", "suprep"])
    ap.add_argument("--fp64", action="store_true")
    ap.add_argument("--out", default=None, help="directory for the .dat files")
    a = ap.parse_args()
    prec = N.FP64 if a.fp64 else N.MIXED
    if a.what == "vw":
        t, r = vw_search(precision=prec)
        out = {"protocol": "OneD_VW.cc MODE2 S1-S2 search", "first_vulnerable_s2_ms": t,
               "timings_in_launch": int(len(r["s2"])), "device_ms": r["device_ms"],
               "cell_steps_per_s": r["cell_steps"] / (r["device_ms"] / 1e3),
               "window_ms": [float(r["s2"][r["vulnerable"]].min()), float(r["s2"][r["vulnerable"]].max())]
               if r["vulnerable"].any() else None}
        if t is not None and a.out:
            write_vw_dat(os.path.join(a.out, "Transmural1D_s2@%.2f.dat" % t), vw_final_cycle(t, precision=prec))
    else:
        r = suprep_sweep(precision=prec, out_dir=a.out)
        out = {"protocol": "SUPREP dose series, LQT1 + ISO1 strand", "device_ms": r["device_ms"],
               "dose_fmol": [x["dose"] for x in r["results"]], "qt_ms": [x["qt"] for x in r["results"]],
               "apd90_median_ms": [float(np.median(x["apd90"])) for x in r["results"]]}
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
