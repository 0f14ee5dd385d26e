"""The shipped surrogate network judged by the FP64 oracle alone, on the CPU:
states of paced endo/epi/M cells (the bench's model) wherever the surrogate
would take them (|dV/dt| <= 1.5 mV/ms), their state after nsub plain steps
against one coarse step of the macro length, and the network's correction
computed by the FP64 reference MLP (oracle/mlp_ref.py, BF16 rounding where the
device rounds).  The correction removes most of the coarse step's error; for a
few slow gates, whose coarse error is already tiny, it does not."""
import json
import os

import numpy as np

from oracle import mlp_ref

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "..", "lqt1_gb300", "data", "tpord_surrogate.npz")
# network order of the 38 evolving states -> reference state index (0..39)
REF_INDEX = [0] + list(range(1, 9)) + [9 + (j if j < 3 else j + 2) for j in range(29)]


def test_network_correction_against_oracle(orc):
    z = np.load(WEIGHTS)
    nsub = int(json.loads(str(z["meta"]))["macro_steps"])
    g, p, i = 0.5, 2.0, 1.5
    m = orc.model("baseline", gks_scale=g, pca_scale=p, gks_iso_scale=i)
    types = [orc.ENDO, orc.EPI, orc.MCELL]
    st = orc.initial_state(-87.5, 3)
    states, cls = [], []
    t = 0.0
    for _ in range(200):                      # 800 ms, a sample every 4 ms
        for _ in range(199):
            orc.cells_update(st, types, m, dt=0.02, ist=np.full(3, -52.0 if t < 2.0 else 0.0), nsteps=1)
            t += 0.02
        v0 = st[:, 0].copy()
        orc.cells_update(st, types, m, dt=0.02, ist=np.zeros(3), nsteps=1)
        t += 0.02
        dv = (st[:, 0] - v0) / 0.02
        for c in range(3):
            if abs(dv[c]) <= 1.5:
                states.append(st[c].copy())
                cls.append(c)
    S = np.array(states)
    cls = np.array(cls)
    assert len(S) > 400
    ty = [types[c] for c in cls]
    fine = orc.cells_update(S.copy(), ty, m, dt=0.02, nsteps=nsub)
    coarse = orc.cells_update(S.copy(), ty, m, dt=0.02 * nsub, nsteps=1)
    D = (fine - coarse)[:, REF_INDEX]
    x = np.zeros((len(S), 48))
    x[:, :38] = S[:, REF_INDEX]
    x[:, 38:41] = (g, p, i)
    x[np.arange(len(S)), 41 + cls] = 1.0          # endo / epi / M one-hot
    xn = np.zeros_like(x)
    xn[:, :44] = (x[:, :44] - z["in_mean"][:44]) * z["in_scale"][:44]
    y = mlp_ref.forward(z["params"], xn, round_bf16=True)["y"]
    corr = y[:, :38] * z["out_scale"][:38]
    ratio = np.sqrt(((corr - D) ** 2).mean(0)) / np.maximum(np.sqrt((D ** 2).mean(0)), 1e-30)
    assert np.median(ratio) < 0.1, ratio
    assert ratio[0] < 0.3, ratio[0]                # V
    assert (ratio < 1.0).sum() >= 32, ratio        # all but a few slow gates improve
