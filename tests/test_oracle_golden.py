"""Pin the CPU oracle against the reference's own outputs (tests/golden/,
made by tests/golden/make_golden.py from the unmodified reference drivers)."""
import json
import os

import numpy as np
import pytest

STRAND_TYPES = np.array([3] * 25 + [4] * 35 + [2] * 40, np.uint8)   # OneD.cc:60-64, 136-200


@pytest.mark.parametrize("variant", ["default", "baseline", "lqt1", "lqt1half", "suprep"])
def test_update_known_answers_bitwise(orc, golden_dir, variant):
    """oracle update() == reference TPORd::update() bit for bit (TPORd.cc:379-1021)."""
    g = np.load(os.path.join(golden_dir, "ref_update_vectors.npz"))
    m = orc.model(variant)
    for steps, key in [(1, "s_out1"), (50, "s_out50")]:
        s = g[f"{variant}__s_in"].copy()
        orc.cells_update(s, g[f"{variant}__types"], m, ist=g[f"{variant}__ist"], dvgap=g[f"{variant}__dvgap"],
                         nsteps=steps)
        ref = g[f"{variant}__{key}"]
        assert np.array_equal(s.view(np.uint64), ref.view(np.uint64)), (
            f"{variant}/{steps}: max diff {np.abs(s - ref).max()}")


def test_single_cell_apd_stats(orc, golden_dir):
    """SingleCell.cc APD statistics, printed to 5 decimals (SingleCell.cc:220-231)."""
    g = json.load(open(os.path.join(golden_dir, "ref_single_cell.json")))
    stats, trace, _ = orc.single_cell_run(orc.MCELL, orc.model("default"), trace_every=50,
                                          trace_cap=200000)
    names = {"rest": "Resting membrane potential", "dvdt_max": "Maximum dV/dt (UpstrokeVelocity_max)",
             "overshoot": "Overshoot", "amplitude": "Amplitude", "apd20": "APD20", "apd25": "APD25",
             "apd50": "APD50", "apd75": "APD75", "apd80": "APD80", "apd90": "APD90"}
    for k, label in names.items():
        assert f"{stats[k]:.5f}" == f"{g['stats'][label]:.5f}", k
    assert abs(stats["apd90"] - 353.94) < 5e-6
    # last two beats, 1 ms samples, printed %4.10f
    v = trace[g["trace_step0"] // g["trace_every"]:]
    np.testing.assert_allclose(v, g["v"], rtol=0, atol=5.1e-11)


def test_strand_first_beat_matches_reference(orc, golden_dir):
    """OneD.cc V samples over the first 1000 ms (CON+ISO1 build)."""
    g = np.load(os.path.join(golden_dir, "ref_oned_default.npz"))
    r = orc.strand_run(STRAND_TYPES, np.full(100, 0.154), orc.model("default"), stop_time=1000.0)
    rows = g["rows"][g["rows"] < len(r["rec"])]
    np.testing.assert_allclose(r["rec"][rows][:, g["cells"]], g["v"][:len(rows)], rtol=0, atol=5.1e-11)
    np.testing.assert_allclose(r["rec_t"][rows], g["t"][:len(rows)], rtol=0, atol=5.1e-11)


@pytest.mark.slow
def test_strand_full_run_cv_and_ecg(orc, golden_dir):
    """1D strand workload (LQT1 GKs x0.5, 2 ms stimulus): V, CV and the
    pseudo-ECG of PlotScript/plot1DECG_compare.py over all 6000 ms."""
    g = np.load(os.path.join(golden_dir, "ref_oned_cfg1.npz"))
    r = orc.strand_run(STRAND_TYPES, np.full(100, 0.154), orc.model("lqt1half"), stim_dur=2.0)
    np.testing.assert_allclose(r["rec"][g["rows"]][:, g["cells"]], g["v"], rtol=0, atol=5.1e-11)
    assert f"{r['cv']:.6g}" == f"{float(g['cv']):.6g}"
    assert abs(r["cv_start"] - float(g["cv_start"])) < 1e-6 and abs(r["cv_end"] - float(g["cv_end"])) < 1e-6
    ecg = np.array([orc.ecg_1d(row) for row in r["rec"][::5]])
    np.testing.assert_allclose(ecg, g["ecg"], rtol=0, atol=1e-9)


def test_stimulus_window_uses_floating_time(orc):
    """OneD.cc:337-338: the window is tested on accumulated `time += dt`."""
    t = 0.0
    on = []
    for _ in range(5000):
        on.append(orc.in_window(t, 1000.0, 50.0, 2.0))
        t += 0.02
    idx = np.nonzero(on)[0]
    assert idx[0] == 2500 and len(idx) in (100, 101)
