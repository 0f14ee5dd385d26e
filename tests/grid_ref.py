"""Oracle-side drivers for grid parity tests: step the CPU oracle grid with the
same stimulus protocol the device applies (OneD.cc:337-338 window on the
accumulated time; S2 on [s2_time, s2_time + s2_duration))."""
import math

import numpy as np


def run_oracle_grid(orc, og, model, nsteps, *, dt=0.02, v0=-87.5, s1_mask=None, bcl=1000.0, s1_start=0.0,
                    s1_dur=2.0, s1_strength=-52.0, s1_beats=0, s2_mask=None, s2_time=-1.0, s2_dur=0.0,
                    s2_strength=0.0, act_thr=-30.0, record_every=0, electrodes=None, ecg_every=0, nthreads=0):
    """Returns final state, activation times (first upward crossing per voxel
    after the first S1 window), V records and ECG samples."""
    state = orc.initial_state(v0, og.n)
    s1t = None if s1_mask is None else s1_mask.reshape(-1)[og.tissue_cell].astype(bool)
    s2t = None if s2_mask is None else s2_mask.reshape(-1)[og.tissue_cell].astype(bool)
    t_act = np.full(og.n, -1.0)
    time = 0.0
    recs, ecg, ecg_t = [], [], []
    for k in range(nsteps):
        ist = np.zeros(og.n)
        if s1t is not None and orc.in_window(time, bcl, s1_start, s1_dur) and (
                s1_beats <= 0 or math.floor(time / bcl) < s1_beats):
            ist[s1t] = s1_strength
        if s2t is not None and s2_time >= 0 and s2_time <= time < s2_time + s2_dur:
            ist[s2t] = s2_strength
        vold = state[:, 0].copy()
        og.step(state, model, dt, ist, nthreads)
        new = (vold < act_thr) & (state[:, 0] >= act_thr) & (t_act < 0)
        t_act[new] = time
        time += dt
        if record_every and (k + 1) % record_every == 0:
            recs.append(state[:, 0].copy())
        if electrodes is not None and ecg_every and (k + 1) % ecg_every == 0:
            ecg.append([og.ecg(state, e) for e in electrodes])
            ecg_t.append(time)
    return dict(state=state, t_act=t_act, rec=np.array(recs), ecg=np.array(ecg), ecg_t=np.array(ecg_t))
