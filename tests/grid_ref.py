"""Oracle-side drivers for grid parity tests: step the CPU oracle grid with the
same stimulus protocol the device applies (OneD.cc:337-338 window on the
accumulated time; S2 on [s2_time, s2_time + s2_duration))."""
import math

import numpy as np


class TissueDetector:
    """APD90 in tissue, restated in FP64 over every voxel at once: at the step
    whose S1 window opens, rest = the V before that step; activation = first
    upward crossing of act_thr (OneD.cc:419-436); overshoot = the largest V
    since activation (tissue rule: the first non-rising step of
    SingleCell.cc:160-198 is kept as the initial overshoot, and later higher V
    raises it); APD90 = first step from at-or-above to at-or-below
    overshoot - 0.9 * (overshoot - rest) (SingleCell.cc:195,211), measured
    from activation.  Times are pre-increment step times."""
    WAIT, RISE, FALL, DONE, IDLE = 1, 2, 3, 4, 0

    def __init__(self, n, act_thr=-30.0):
        self.thr = act_thr
        self.phase = np.zeros(n, np.int8)
        self.vrest = np.zeros(n)
        self.vpeak = np.zeros(n)
        self.t_act = np.full(n, -1.0)
        self.apd90 = np.full(n, -1.0)

    def open_cycle(self, vold):
        self.vrest[:] = vold
        self.vpeak[:] = vold
        self.phase[:] = self.WAIT

    def step(self, vold, vnew, time):
        ph = self.phase
        act = (ph == self.WAIT) & (vold < self.thr) & (vnew >= self.thr)
        rise = ph == self.RISE
        fall = ph == self.FALL
        up = rise & (vnew > vold)
        top = rise & ~(vnew > vold)
        higher = fall & (vnew > self.vpeak)
        amp = self.vpeak - self.vrest
        thr90 = self.vpeak - 0.9 * amp
        done = fall & ~higher & (vnew <= thr90) & (vold >= thr90)
        self.vpeak[up] = vnew[up]
        self.vpeak[top] = vold[top]
        self.vpeak[higher] = vnew[higher]
        self.apd90[done] = time - self.t_act[done]
        self.t_act[act] = time
        self.vpeak[act] = vnew[act]
        ph[top] = self.FALL
        ph[done] = self.DONE
        ph[act] = self.RISE


def run_oracle_grid(orc, og, model, nsteps, *, dt=0.02, v0=-87.5, s1_mask=None, bcl=1000.0, s1_start=0.0,
                    s1_dur=2.0, s1_strength=-52.0, s1_beats=0, s2_mask=None, s2_time=-1.0, s2_dur=0.0,
                    s2_strength=0.0, act_thr=-30.0, record_every=0, electrodes=None, ecg_every=0, nthreads=0,
                    detect=False):
    """Returns final state, activation times (first upward crossing per voxel
    after the first S1 window), V records and ECG samples; with detect, also
    the tissue APD90 of the last completed cycle (TissueDetector)."""
    state = orc.initial_state(v0, og.n)
    det = TissueDetector(og.n, act_thr) if detect else None
    was_on = False
    s1t = None if s1_mask is None else s1_mask.reshape(-1)[og.tissue_cell].astype(bool)
    s2t = None if s2_mask is None else s2_mask.reshape(-1)[og.tissue_cell].astype(bool)
    t_act = np.full(og.n, -1.0)
    time = 0.0
    recs, ecg, ecg_t = [], [], []
    for k in range(nsteps):
        ist = np.zeros(og.n)
        s1_on = s1t is not None and orc.in_window(time, bcl, s1_start, s1_dur) and (
            s1_beats <= 0 or math.floor(time / bcl) < s1_beats)
        if s1_on:
            ist[s1t] = s1_strength
        if s2t is not None and s2_time >= 0 and s2_time <= time < s2_time + s2_dur:
            ist[s2t] = s2_strength
        vold = state[:, 0].copy()
        if det is not None and s1_on and not was_on:
            det.open_cycle(vold)
        was_on = s1_on
        og.step(state, model, dt, ist, nthreads)
        new = (vold < act_thr) & (state[:, 0] >= act_thr) & (t_act < 0)
        t_act[new] = time
        if det is not None:
            det.step(vold, state[:, 0], time)
        time += dt
        if record_every and (k + 1) % record_every == 0:
            recs.append(state[:, 0].copy())
        if electrodes is not None and ecg_every and (k + 1) % ecg_every == 0:
            ecg.append([og.ecg(state, e) for e in electrodes])
            ecg_t.append(time)
    out = dict(state=state, t_act=t_act, rec=np.array(recs), ecg=np.array(ecg), ecg_t=np.array(ecg_t))
    if det is not None:
        out.update(apd90=det.apd90, t_act_last=det.t_act)
    return out
