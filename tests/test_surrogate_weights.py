"""The shipped surrogate weights file, checked on the CPU: the parameter block
has the network's size and is finite, the normalisation and residual bounds
are usable, the macro length divides the 50-step graph span, and the file
records the held-out accuracy and the tissue-validation selection it was
shipped on."""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "..", "lqt1_gb300", "data", "tpord_surrogate.npz")
IN, HID, OUT, N_STATE = 48, 128, 48, 38


def _load():
    z = np.load(WEIGHTS)
    return z, json.loads(str(z["meta"]))


def test_parameter_block_and_normalisation():
    z, _ = _load()
    p = z["params"]
    assert p.dtype == np.float32
    assert p.size == HID * IN + HID + HID * HID + HID + OUT * HID + OUT
    assert np.isfinite(p).all()
    assert z["in_mean"].shape == (IN,) and z["in_scale"].shape == (IN,) and z["out_scale"].shape == (OUT,)
    assert np.isfinite(z["in_mean"]).all() and (z["in_scale"] > 0).all()
    assert (z["out_scale"][:N_STATE] > 0).all()
    b = z["out_bound"][:N_STATE]
    assert np.isfinite(b).all() and (b > 0).all()


def test_macro_length_and_recorded_accuracy():
    _, m = _load()
    nsub = int(m["macro_steps"])
    assert 1 <= nsub <= 50 and 50 % nsub == 0
    assert m["dt"] == 0.02
    r = np.asarray(m["val_rmse"]) / np.maximum(np.asarray(m["val_zero_rmse"]), 1e-30)
    assert r.shape == (N_STATE,)
    assert np.median(r) < 0.15 and r[0] < 0.5 and (r < 1.0).all()
    assert len(m["state_names"]) == N_STATE and m["state_names"][0] == "v"


def test_selection_record():
    _, m = _load()
    sel = m["selection"]
    c = sel["candidates"]
    assert len(c) >= 2 and "validation sheet" in sel["rule"]
    # the shipped network is the least biased of the recorded candidates
    assert abs(c[0]["apd_bias_ms"]) == min(abs(x["apd_bias_ms"]) for x in c)
