"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs only where the reference sources are present (they are absent on the GPU
host): builds the reference with oracle/build_ref.sh, runs its unmodified
drivers (SingleCell.cc, OneD.cc) and a scenario variant of OneD.cc, calls its
TPORd::update() through oracle/ref_harness.inc, and writes compact fixtures:

  ref_update_vectors.npz   known-answer vectors of TPORd::update() per scenario
  ref_single_cell.json     SingleCell.cc APD statistics + last-beat V samples
  ref_oned_default.npz     OneD.cc (CON+ISO1, 1 ms stimulus) V samples, CV
  ref_oned_cfg1.npz        OneD.cc with LQT1 GKs x0.5, ISO1 off, 2 ms stimulus
                           (the 1D strand workload), V samples, CV, pseudo-ECG

Usage: python tests/golden/make_golden.py REFERENCE_DIR
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import orc  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LQT_REFERENCE")
if not REF:
    sys.exit("usage: make_golden.py REFERENCE_DIR (a checkout of ShugangZhang/LQT1), or set LQT_REFERENCE")
BIN = os.path.join(ROOT, "oracle", "_ref")


def build():
    subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh"), REF], check=True)


def update_vectors():
    """Reference TPORd::update() on seeded random states, 1 and 50 steps."""
    out = {}
    for k, variant in enumerate(["default", "baseline", "lqt1", "lqt1half", "suprep"]):
        n = 64
        rng = np.random.default_rng(100 + k)
        s_in = orc.random_states(n, seed=200 + k)
        types = rng.integers(0, 5, n).astype(np.uint8)
        ist = np.where(rng.random(n) < 0.25, -52.0, 0.0)
        dvgap = rng.normal(0.0, 5.0, n)
        s1 = orc.ref_update(s_in.copy(), types, variant, ist=ist, dvgap=dvgap, nsteps=1)
        s50 = orc.ref_update(s_in.copy(), types, variant, ist=ist, dvgap=dvgap, nsteps=50)
        for name, arr in [("s_in", s_in), ("types", types), ("ist", ist), ("dvgap", dvgap), ("s_out1", s1),
                          ("s_out50", s50)]:
            out[f"{variant}__{name}"] = arr
    np.savez_compressed(os.path.join(OUT, "ref_update_vectors.npz"), **out)


def single_cell(work):
    run = os.path.join(work, "sc")
    os.makedirs(os.path.join(run, "Outputs"))
    log = subprocess.run([os.path.join(BIN, "model_single_cell")], cwd=run, check=True, capture_output=True,
                         text=True).stdout
    stats = {}
    for line in open(os.path.join(run, "Outputs", "VentriSingleCellStats.dat")):
        key, val = line.split("=")
        stats[key.strip()] = float(val.split()[0])
    # V after every step (SingleCell.cc:113-139, one line per step); keep every
    # 50th (1 ms) of the last two beats: steps 4,900,000 .. 4,999,999.
    t, v = [], []
    with open(os.path.join(run, "Outputs", "VentriSingleCellResults_LQT1_ISO_MCELL.dat")) as f:
        for i, line in enumerate(f):
            if i >= 4_900_000 and i % 50 == 0:
                a, b = line.split("\t")[:2]
                t.append(float(a))
                v.append(float(b))
    json.dump({"driver": "SingleCell.cc (unmodified; MCELL, CON+ISO1, BCL 1000, 100 beats, -53 x 1 ms)",
               "stats": stats, "stdout_tail": log.strip().splitlines()[-13:], "trace_step0": 4_900_000,
               "trace_every": 50, "t": t, "v": v},
              open(os.path.join(OUT, "ref_single_cell.json"), "w"), indent=0)


def ecg_restated(vrows, dx=0.15, x0=20 + 15):
    """PlotScript/plot1DECG_compare.py:82-105 restated with numpy (that script
    needs matplotlib, which is absent): phi = sum_i -dV_i / (x_i - x0)^2 with
    one-sided differences at the ends and half central differences inside."""
    n = vrows.shape[1]
    x = np.arange(n) * dx - x0
    dv = np.empty_like(vrows)
    dv[:, 0] = vrows[:, 1] - vrows[:, 0]
    dv[:, -1] = vrows[:, -1] - vrows[:, -2]
    dv[:, 1:-1] = (vrows[:, 2:] - vrows[:, :-2]) / 2
    return (-dv / (x * x)).sum(axis=1)


def oned(work, exe, datname, outname, desc):
    run = os.path.join(work, outname)
    os.makedirs(os.path.join(run, "Outputs"))
    log = subprocess.run([os.path.join(BIN, exe)], cwd=run, check=True, capture_output=True, text=True).stdout
    m = re.search(r"start = ([-\d.e+]+)", log)
    cv_start = float(m.group(1))
    cv_end = float(re.search(r"end = ([-\d.e+]+)", log).group(1))
    cv = float(re.search(r"CV = ([-\d.e+]+) m/s", log).group(1))
    data = np.loadtxt(os.path.join(run, "Outputs", datname))
    t, v = data[:, 0], data[:, 1:]
    ecg = ecg_restated(v)
    cells = np.arange(0, 100, 5)
    rows = np.arange(0, len(t), 25)  # every 5 ms (rows are 0.2 ms apart, OneD.cc:402)
    np.savez_compressed(os.path.join(OUT, outname + ".npz"), t=t[rows], v=v[np.ix_(rows, cells)], cells=cells,
                        rows=rows, cv=cv, cv_start=cv_start, cv_end=cv_end, ecg_t=t[::5], ecg=ecg[::5],
                        v_last=v[-1], desc=desc)


def main():
    build()
    update_vectors()
    with tempfile.TemporaryDirectory() as work:
        single_cell(work)
        oned(work, "model_oned", "VentOneDResults_CON_ISO.dat", "ref_oned_default",
             "OneD.cc unmodified: CON+ISO1, 25 endo/35 M/40 epi, 1 ms x -52 pA/pF, BCL 1000, 6000 ms")
        oned(work, "model_oned_cfg1", "VentOneDResults_LQT1.dat", "ref_oned_cfg1",
             "OneD.cc with LQT1 GKs x0.5, ISO1 off, 2 ms stimulus (oracle/build_ref.sh)")
    print("fixtures written to", OUT)


if __name__ == "__main__":
    main()
