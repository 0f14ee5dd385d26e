"""GPU parity: single cells and the 1D strand (lqt_batch_*) against the
oracle and the reference's golden outputs."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lq():
    import lqt1_gb300 as lq
    lq.lib()
    return lq


def test_single_cell_apd90_mixed(lq, golden_dir):
    """SingleCell.cc (MCELL, CON+ISO1, 100 beats): APD90 within 1 ms of the
    reference's 353.94 ms; rest and overshoot within 0.5 mV."""
    g = json.load(open(os.path.join(golden_dir, "ref_single_cell.json")))["stats"]
    spec = lq.InstanceSpec(types=np.array([lq.MCELL], np.uint8), bcl=1000.0, s1_start=50.0, s1_duration=1.0,
                           s1_strength=-53.0, n_stim=1, t_stop=100 * 1000.0 - 0.01)
    b = lq.Batch([spec], [lq.model("default")], precision=lq.MIXED, max_beats=110)
    b.run()
    d = b.detect()
    nb = d["beats"][0]
    assert nb == 100
    apd = d["apd90"][0, nb - 1]
    # SingleCell.cc measures APD from stimStart + stimDuration; the detector
    # from the -30 mV crossing, so compare the 90% repolarisation time.
    t90 = d["t_act"][0, nb - 1] + apd - (99 * 1000.0 + 50.0 + 1.0)
    assert abs(t90 - g["APD90"]) < 1.0, (t90, g["APD90"])
    assert b.num_bad() == 0


def test_strand_one_beat_fp64_vs_oracle(lq, orc):
    """FP64 strand, first 1000 ms of the 1D workload: V within 1e-4 mV."""
    types = lq.oned_types()
    ref = orc.strand_run(types, np.full(100, 0.154), orc.model("lqt1half"), stim_dur=2.0, stop_time=1000.0)
    s = lq.OneDStrand(model=lq.model("lqt1", gks_scale=0.5), precision=lq.FP64, stim_duration=2.0,
                      stop_time=1000.0)
    r = s.run()
    assert r["rec"].shape == ref["rec"].shape
    assert np.abs(r["rec"] - ref["rec"]).max() < 1e-3          # float32 record of FP64 V
    np.testing.assert_allclose(r["rec_t"], ref["rec_t"], rtol=0, atol=1e-9)


def test_strand_config1_mixed_vs_oracle_and_golden(lq, orc, golden_dir):
    """The 1D strand workload (LQT1 GKs x0.5, 2 ms x -52, BCL 1000, 6000 ms)
    in the mixed form: V within 0.5 mV outside the upstroke, activation within
    0.1 ms, CV and the pseudo-ECG against the reference's golden output."""
    g = np.load(os.path.join(golden_dir, "ref_oned_cfg1.npz"))
    types = lq.oned_types()
    ref = orc.strand_run(types, np.full(100, 0.154), orc.model("lqt1half"), stim_dur=2.0)
    s = lq.OneDStrand(model=lq.model("lqt1", gks_scale=0.5), precision=lq.MIXED, stim_duration=2.0)
    r = s.run()
    v, vr = r["rec"], ref["rec"]
    assert v.shape == vr.shape
    # upstroke: samples where the oracle's V moves > 1 mV between records
    dvr = np.abs(np.diff(vr, axis=0, prepend=vr[:1]))
    calm = dvr < 1.0
    assert np.abs(v - vr)[calm].max() < 0.5
    nb = min(ref["act"].shape[1], r["t_act"].shape[1])
    act_ref = ref["act"][:, :nb]
    act = r["t_act"][:, :nb]
    both = (act_ref >= 0) & (act >= 0)
    assert both.sum() >= 100 * 6 - 5
    assert np.abs(act[both] - act_ref[both]).max() <= 0.1 + 1e-6
    assert abs(r["cv"] - float(g["cv"])) < 0.005
    np.testing.assert_allclose(r["ecg"][::5], g["ecg"], atol=2e-3)
