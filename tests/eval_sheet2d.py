"""Accuracy evaluations of the mixed form against the FP64 forms on the GPU and
the CPU oracle, on the 2D sheet workload.

  python tests/eval_sheet2d.py sheet2d [--n 600] [--t-end 2000] [--seed 7]

2D sheet: n x n tissue at 0.15 mm, isotropic D = 0.154, bands 30/35/35 %
endo/M/epi; one S1 plane wave from the x = 0 edge at t = 0 (2 ms x -52); S2 on
the quadrant x < n/2, y < n/2 (3 ms x -104 pA/pF, the S2 strength of
OneD_VW.cc:68-70) at a seeded coupling interval U[300, 360] ms.  Both forms run
on the GPU; maps of activation time (S1 wave and last wave) and V are
compared.  A reduced sheet is also checked against the CPU oracle.
Prints one JSON object.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import lqt1_gb300 as lq  # noqa: E402


def run_sheet(n, t_end, ci, precision, model, t_mid):
    sh = lq.geometry.sheet(n, n, s1_cols=3)
    sim = lq.Sim(sh.types, 0.15, precision=precision, model=model)
    sim.set_protocol(bcl=1000.0, s1_mask=sh.s1_mask, s1_start=0.0, s1_duration=2.0, s1_strength=-52.0, s1_beats=1,
                     s2_time=ci, s2_duration=3.0, s2_strength=-104.0, s2_mask=sh.s2_mask)
    t0 = time.perf_counter()
    sim.step(int(round(t_mid / 0.02)))
    d_mid = sim.detect()
    v_mid = sim.get_v(as_double=True)
    sim.step(int(round((t_end - t_mid) / 0.02)))
    d_end = sim.detect()
    v_end = sim.get_v(as_double=True)
    wall = time.perf_counter() - t0
    return dict(t_act_s1=d_mid["t_act"], v_mid=v_mid, t_act_end=d_end["t_act"], apd_end=d_end["apd90"], v_end=v_end,
                wall_s=wall, n=sim.n, nbad=sim.check())


def err_stats(a, b, mask=None):
    d = np.abs(np.asarray(a, np.float64) - np.asarray(b, np.float64))
    if mask is not None:
        d = d[mask]
    if d.size == 0:
        return None
    return {"max": float(d.max()), "p99": float(np.percentile(d, 99)), "mean": float(d.mean()), "n": int(d.size)}


def sheet2d(args):
    rng = np.random.default_rng(args.seed)
    ci = float(rng.uniform(300.0, 360.0))
    model = lq.model("lqt1", gks_scale=0.5)
    out = {"workload": f"2d-sheet {args.n}x{args.n} @0.15mm", "s2_coupling_ms": ci, "t_end_ms": args.t_end}
    t_mid = ci - 1.0
    mx = run_sheet(args.n, args.t_end, ci, lq.MIXED, model, t_mid)
    f64 = run_sheet(args.n, args.t_end, ci, lq.FP64, model, t_mid)
    act = (mx["t_act_s1"] >= 0) & (f64["t_act_s1"] >= 0)
    out["mixed_vs_fp64_gpu"] = {
        "s1_activation_ms": err_stats(mx["t_act_s1"], f64["t_act_s1"], act),
        "s1_activated_both": int(act.sum()), "tissue": int(mx["n"]),
        "s1_within_0.1ms": float((np.abs(mx["t_act_s1"] - f64["t_act_s1"])[act] <= 0.1).mean()),
        "v_at_s2_minus_1ms_mV": err_stats(mx["v_mid"], f64["v_mid"]),
        "last_activation_ms": err_stats(mx["t_act_end"], f64["t_act_end"],
                                        (mx["t_act_end"] >= 0) & (f64["t_act_end"] >= 0)),
        "apd90_last_ms": err_stats(mx["apd_end"], f64["apd_end"], (mx["apd_end"] >= 0) & (f64["apd_end"] >= 0)),
        "v_end_mV": err_stats(mx["v_end"], f64["v_end"]),
        "wall_s": {"mixed": mx["wall_s"], "fp64": f64["wall_s"]},
        "blowups": {"mixed": mx["nbad"], "fp64": f64["nbad"]},
    }
    # reduced sheet against the CPU oracle (FP64, same protocol, S1 wave only)
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from oracle import orc
    nr, tr = args.n_cpu, args.t_cpu
    sh = lq.geometry.sheet(nr, nr, s1_cols=3)
    og = orc.Grid(sh.types, 0.15)
    st = orc.initial_state(-87.5, og.n)
    s1t = sh.s1_mask.reshape(-1)[og.tissue_cell].astype(bool)
    t_act = np.full(og.n, -1.0)
    tt = 0.0
    for _ in range(int(round(tr / 0.02))):
        ist = np.where(s1t & orc.in_window(tt, 1000.0, 0.0, 2.0), -52.0, 0.0)
        vold = st[:, 0].copy()
        og.step(st, orc.model("lqt1half"), 0.02, ist)
        new = (vold < -30) & (st[:, 0] >= -30) & (t_act < 0)
        t_act[new] = tt
        tt += 0.02
    res = {}
    for name, prec in (("mixed", lq.MIXED), ("fp64", lq.FP64)):
        sim = lq.Sim(sh.types, 0.15, precision=prec, model=model)
        sim.set_protocol(bcl=1000.0, s1_mask=sh.s1_mask, s1_start=0.0, s1_duration=2.0, s1_strength=-52.0, s1_beats=1)
        sim.step(int(round(tr / 0.02)))
        d = sim.detect()
        both = (d["t_act"] >= 0) & (t_act >= 0)
        res[name] = {"activation_ms": err_stats(d["t_act"], t_act, both), "activated": int(both.sum()),
                     "v_mV": err_stats(sim.get_v(as_double=True), st[:, 0])}
    out["vs_cpu_oracle"] = {"sheet": f"{nr}x{nr}", "t_ms": tr, **res}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["sheet2d"])
    ap.add_argument("--n", type=int, default=600)
    ap.add_argument("--t-end", type=float, default=2000.0)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--n-cpu", type=int, default=100)
    ap.add_argument("--t-cpu", type=float, default=150.0)
    args = ap.parse_args()
    print(json.dumps(sheet2d(args)), flush=True)


if __name__ == "__main__":
    main()
