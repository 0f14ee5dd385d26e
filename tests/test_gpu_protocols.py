"""The reference drivers' protocols as batched launches, against the FP64
oracle: the S1-S2 vulnerable-window search of OneD_VW.cc, the SUPREP dose
series, SingleCell.cc's current output, and the VTK snapshots of GPU3D.cu."""
import os

import numpy as np
import pytest

from oracle import io_ref

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lq():
    import lqt1_gb300 as lq
    lq.lib()
    return lq


def test_vw_trials_match_oracle(lq, orc):
    """maxEndo / maxEpi of OneD_VW.cc trials (2 S1 cycles, S2 at three
    coupling intervals), FP64 batch against the FP64 oracle; the mixed form
    reaches the same verdicts."""
    s2 = np.array([240.0, 300.0, 360.0])
    types = lq.protocols.vw_types()
    coeff = lq.protocols.vw_coeff()
    r64 = lq.protocols.vulnerable_window(s2, precision=lq.FP64, num_s1=2)
    rmx = lq.protocols.vulnerable_window(s2, precision=lq.MIXED, num_s1=2)
    for i, t in enumerate(s2):
        me, mp = orc.vw_trial(types, coeff, orc.model("default"), t, num_s1=2)
        assert abs(r64["max_endo"][i] - me) < 1e-3 and abs(r64["max_epi"][i] - mp) < 1e-3, (t, me, mp)
        assert abs(rmx["max_endo"][i] - me) < 0.5 and abs(rmx["max_epi"][i] - mp) < 0.5, (t, me, mp)
    np.testing.assert_array_equal(r64["vulnerable"], rmx["vulnerable"])


def test_vw_search_finds_the_oracles_window(lq, orc):
    """MODE2 search (S2 timings upward in 0.1 ms steps) as batched launches,
    from 200 ms so that the window's opening lies inside the scan.  The mixed
    form scans 1000 timings in one launch; the FP64 batch and the oracle agree
    on the edges: vulnerable at the first and the last timing of the window,
    not 0.1 ms outside either."""
    t_mx, r_mx = lq.protocols.vw_search(start=200.0, step=0.1, batch=1000, max_batches=1, precision=lq.MIXED)
    assert t_mx is not None and t_mx > 200.0
    vul = r_mx["s2"][r_mx["vulnerable"]]
    lo = round(t_mx - 1.0, 1)
    t64, r64 = lq.protocols.vw_search(start=lo, step=0.1, batch=21, max_batches=1, precision=lq.FP64)
    assert t64 is not None and abs(t64 - t_mx) <= 0.5
    hi_mx = float(vul.max())
    r64b = lq.protocols.vulnerable_window(np.round(hi_mx + 0.1 * np.arange(-10, 11), 1), precision=lq.FP64)
    hi64 = float(r64b["s2"][r64b["vulnerable"]].max())
    assert abs(hi64 - hi_mx) <= 0.5
    types = lq.protocols.vw_types()
    coeff = lq.protocols.vw_coeff()
    m = orc.model("default")
    for t, inside in ((t64, True), (round(t64 - 0.1, 1), False), (hi64, True), (round(hi64 + 0.1, 1), False)):
        me, mp = orc.vw_trial(types, coeff, m, t)
        assert ((me + 10) * (mp + 10) <= 0) == inside, (t, me, mp)


def test_vw_final_cycle_file(lq, orc, tmp_path):
    """The Transmural1D_s2@<t>.dat rows: V of every cell every 50 steps of the
    last cycle, in the reference's format."""
    rows = lq.protocols.vw_final_cycle(300.0, precision=lq.FP64, num_s1=2)
    _, _, ref = orc.vw_trial(lq.protocols.vw_types(), lq.protocols.vw_coeff(), orc.model("default"), 300.0,
                             num_s1=2, record=True)
    assert rows.shape == ref.shape == (1000, 100)
    assert np.abs(rows - ref).max() < 1e-3
    p = tmp_path / "Transmural1D_s2@300.00.dat"
    lq.protocols.write_vw_dat(str(p), rows)
    assert p.read_text() == io_ref.dat_text(rows)


def test_suprep_sweep_matches_oracle(lq, orc):
    """Doses 0 and 150 fmol of the LQT1 + ISO1 strand: pseudo-ECG and its QT
    against the oracle strand run (OneD.cc) with the same ECG sum; SUPREP
    restores IKs, so QT and APD90 shorten with dose."""
    r = lq.protocols.suprep_sweep(doses=(0, 150), precision=lq.FP64)["results"]
    for res in r:
        m = orc.model("default", gks_scale=0.05, suprep_dose=res["dose"])
        ref = orc.strand_run(lq.oned_types(), np.full(100, 0.154), m, rec_every=10)
        ecg = np.array([orc.ecg_1d(v) for v in ref["rec"]])
        np.testing.assert_allclose(res["t"], ref["rec_t"], atol=1e-9)
        assert np.abs(res["ecg"] - ecg).max() < 1e-6 * max(1.0, np.abs(ecg).max())
        qt, _ = lq.protocols.qt_from_ecg(ref["rec_t"], ecg, 4050.0, 1000.0)
        assert abs(res["qt"] - qt) < 0.5, (res["dose"], res["qt"], qt)
    assert r[1]["qt"] < r[0]["qt"] - 5.0
    assert np.median(r[1]["apd90"]) < np.median(r[0]["apd90"])


def test_single_cell_currents_record(lq, orc, tmp_path):
    """SingleCell.cc's file: time, V, ICaL, IKs every step, from a batched
    single-cell instance, against orc_update's reported currents."""
    import ctypes as C
    m = lq.model("default")
    spec = lq.InstanceSpec(types=np.array([lq.MCELL], np.uint8), bcl=1000.0, s1_start=50.0, s1_duration=1.0,
                           s1_strength=-53.0, n_stim=1, t_stop=400.0, record=True, currents=True)
    b = lq.Batch([spec], [m], precision=lq.FP64, rec_every=1)
    b.run()
    rec = b.record(0)
    b.close()
    # oracle: the same stimulus windows (OneD.cc:337-338 on floating time)
    L = orc.lib()

    class Aux(C.Structure):
        _fields_ = [(k, C.c_double) for k in ("dvdt", "iion", "ina", "inal", "ito", "ical", "ikr", "iks", "ik1",
                                              "inaca", "inak")]
    s = orc.initial_state(-87.5)[0].copy()
    om = orc.model("default")
    aux = Aux()
    L.orc_update.argtypes = [C.c_void_p, C.c_int, C.POINTER(orc.Model), C.c_double, C.c_double, C.c_double,
                             C.c_void_p]
    t, rows = 0.0, []
    while t <= 400.0 + 1e-12 and len(rows) < len(rec["t"]):
        ist = -53.0 if orc.in_window(t, 1000.0, 50.0, 1.0) else 0.0
        L.orc_update(s.ctypes.data, orc.MCELL, C.byref(om), 0.02, ist, 0.0, C.addressof(aux))
        rows.append((t, s[0], aux.ical, aux.iks))
        t += 0.02
    ref = np.array(rows)
    n = min(len(ref), len(rec["t"]))
    got = np.column_stack([rec["t"], rec["v"][:, 0], rec["ical"], rec["iks"]])[:n]
    np.testing.assert_allclose(got[:, 0], ref[:n, 0], atol=1e-9)
    assert np.abs(got[:, 1] - ref[:n, 1]).max() < 1e-4
    assert np.abs(got[:, 2] - ref[:n, 2]).max() < 1e-4
    assert np.abs(got[:, 3] - ref[:n, 3]).max() < 1e-6
    p = tmp_path / "VentSingleCellResults.dat"
    lq.protocols.write_single_cell_dat(str(p), *got.T)
    assert p.read_text() == io_ref.dat_text(got)


def test_vtk_snapshots_of_a_ventricle(lq, tmp_path):
    """Device lattice sampling equals the gathered V; the asynchronous writer
    produces the reference's VTK layout while the simulation steps on."""
    v = lq.geometry.ventricle(nx=44, ny=44, nz=50, dx=0.2, a_out=4.0, c_out=8.0, wall=2.0, z_base=9.0,
                              island_radius=1.5, stim_radius=1.2)
    sim = lq.Sim(v.types, 0.2, fibre=v.fibre, precision=lq.MIXED, model="lqt1")
    sim.set_protocol(bcl=800.0, s1_mask=v.s1_mask, s1_start=0.0, s1_duration=2.0, s1_strength=-52.0)
    sim.step(500)
    vg = sim.v_grid(fill=np.nan)
    tissue = v.types != 255
    for stride in (1, 3):
        smp = sim.sample_v(stride)
        vv = np.where(tissue, vg, -100.0)[::stride, ::stride, ::stride].transpose(2, 1, 0).reshape(-1)
        np.testing.assert_array_equal(smp, vv)
    paths = []
    with sim.vtk_writer(stride=3, nbuf=2) as w:
        for i in range(4):
            p = tmp_path / f"ap_{i}.vtk"
            w.submit(str(p))
            paths.append((p, sim.sample_v(3)))
            sim.step(50)
    # every file against the restatement of the reference loop, from the
    # samples taken at the moment of its submission
    for p, smp in paths:
        assert os.path.exists(p)
        grid = np.zeros(v.types.shape)
        sub = smp.reshape(tuple(-(-np.array(v.types.shape[::-1]) // 3)))     # (z, y, x)
        grid[::3, ::3, ::3] = sub.transpose(2, 1, 0)
        assert p.read_text() == io_ref.vtk_text(grid, tissue, 3)
    assert paths[0][0].read_text() != paths[-1][0].read_text()
