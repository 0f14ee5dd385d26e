"""GPU parity of the 2D/3D/1D tissue path (lqt_sim_*) against the CPU oracle."""
import numpy as np
import pytest

from grid_ref import run_oracle_grid

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lq():
    import lqt1_gb300 as lq
    lq.lib()
    return lq


def small_sheet(lq, n=40):
    """Anisotropic 2D sheet: fibre angle varies along y (exercises the
    D-gradient terms of new_11.cu:383-414)."""
    sh = lq.geometry.sheet(n, n, s1_cols=3)
    nx, ny = sh.types.shape
    ang = np.linspace(-1.0, 1.0, ny)[None, :].repeat(nx, 0)
    fib = np.zeros((nx, ny, 1, 3), np.float32)
    fib[..., 0, 0] = np.cos(ang)
    fib[..., 0, 1] = np.sin(ang)
    return sh, fib


def small_ventricle(lq):
    return lq.geometry.ventricle(nx=44, ny=44, nz=50, dx=0.2, a_out=4.0, c_out=8.0, wall=2.0, z_base=9.0,
                                 island_radius=1.5, stim_radius=1.2)


@pytest.mark.parametrize("case", ["sheet", "ventricle"])
def test_fp64_grid_matches_oracle(lq, orc, case):
    """FP64 form: 300 steps with an S1 stimulus; every state of every voxel
    against the oracle's grid step (mirror map, tensor, stimulus, TPORd)."""
    if case == "sheet":
        sh, fib = small_sheet(lq)
        types, s1, fibre, dx = sh.types, sh.s1_mask, fib.reshape(sh.types.shape + (3,)), 0.15
    else:
        v = small_ventricle(lq)
        types, s1, fibre, dx = v.types, v.s1_mask, v.fibre, 0.2
    m = "lqt1"
    og = orc.Grid(types, dx, fibre=fibre, d_f=0.154, d_t=0.0385)
    ref = run_oracle_grid(orc, og, orc.model(m), 300, s1_mask=s1, s1_dur=2.0)
    sim = lq.Sim(types, dx, fibre=fibre, precision=lq.FP64, model=m)
    sim.set_protocol(bcl=1000.0, s1_mask=s1, s1_start=0.0, s1_duration=2.0, s1_strength=-52.0)
    sim.step(300)
    got = sim.get_state()
    assert np.isfinite(got).all()
    # last-bit differences of CUDA vs glibc exp/log, amplified through the upstroke
    # (V is compared in absolute terms: it crosses 0 mV in the upstroke)
    assert np.abs(got[:, 0] - ref["state"][:, 0]).max() < 1e-4
    np.testing.assert_allclose(got[:, 1:], ref["state"][:, 1:], rtol=2e-5, atol=1e-8)
    assert sim.check() == 0


def test_mixed_sheet_propagation_vs_oracle(lq, orc):
    """Mixed form on the anisotropic sheet over 60 ms: V within 0.5 mV outside
    the upstroke, activation times within 0.1 ms, ECG within 1%."""
    sh, fib = small_sheet(lq, 60)
    fibre = fib.reshape(sh.types.shape + (3,))
    og = orc.Grid(sh.types, 0.15, fibre=fibre)
    el = [np.array([-3.0, 4.0, 2.0]), np.array([12.0, 4.5, -1.0])]
    nsteps = 3000
    ref = run_oracle_grid(orc, og, orc.model("default"), nsteps, s1_mask=sh.s1_mask, s1_dur=2.0,
                          record_every=50, electrodes=el, ecg_every=50)
    sim = lq.Sim(sh.types, 0.15, fibre=fibre, precision=lq.MIXED, model="default")
    sim.set_protocol(bcl=1000.0, s1_mask=sh.s1_mask, s1_start=0.0, s1_duration=2.0, s1_strength=-52.0)
    sim.set_electrodes(np.array(el), every=50)
    recs = []
    for _ in range(nsteps // 50):
        sim.step(50)
        recs.append(sim.get_v(as_double=True))
    recs = np.array(recs)
    dref = np.abs(np.diff(ref["rec"], axis=0, prepend=ref["rec"][:1]))
    calm = dref < 1.0
    assert np.abs(recs - ref["rec"])[calm].max() < 0.5
    det = sim.detect()
    both = (det["t_act"] >= 0) & (ref["t_act"] >= 0)
    assert both.sum() == (ref["t_act"] >= 0).sum() > 0.9 * og.n
    assert np.abs(det["t_act"][both] - ref["t_act"][both]).max() <= 0.1 + 1e-4
    phi, t = sim.ecg()
    assert phi.shape == ref["ecg"].shape
    np.testing.assert_allclose(t, ref["ecg_t"], atol=1e-9)
    scale = np.abs(ref["ecg"]).max(axis=0)
    assert (np.abs(phi - ref["ecg"]).max(axis=0) <= 0.01 * scale + 1e-6).all()


def test_mixed_ventricle_vs_oracle(lq, orc):
    """Mixed form on a small ventricle-shaped shell (fibres rotating through the
    wall, apical stimulus) over 40 ms."""
    v = small_ventricle(lq)
    og = orc.Grid(v.types, 0.2, fibre=v.fibre)
    nsteps = 2000
    ref = run_oracle_grid(orc, og, orc.model("lqt1half"), nsteps, s1_mask=v.s1_mask, s1_dur=2.0,
                          record_every=100)
    sim = lq.Sim(v.types, 0.2, fibre=v.fibre, precision=lq.MIXED, model=lq.model("lqt1", gks_scale=0.5))
    sim.set_protocol(bcl=800.0, s1_mask=v.s1_mask, s1_start=0.0, s1_duration=2.0, s1_strength=-52.0)
    recs = []
    for _ in range(nsteps // 100):
        sim.step(100)
        recs.append(sim.get_v(as_double=True))
    recs = np.array(recs)
    dref = np.abs(np.diff(ref["rec"], axis=0, prepend=ref["rec"][:1]))
    calm = dref < 1.0
    assert np.abs(recs - ref["rec"])[calm].max() < 0.5
    det = sim.detect()
    both = (det["t_act"] >= 0) & (ref["t_act"] >= 0)
    assert both.sum() == (ref["t_act"] >= 0).sum()
    assert np.abs(det["t_act"][both] - ref["t_act"][both]).max() <= 0.1 + 1e-4


def test_sim_1d_matches_oracle_strand(lq, orc):
    """A 1D grid through lqt_sim (OneD.cc diffusion incl. the dD/dx term with a
    non-uniform coefficient) against the oracle strand driver, FP64, 500 ms."""
    types = lq.oned_types()
    coeff = np.full(100, 0.154)
    coeff[59] = 0.2 * 0.154          # the OneD_VW.cc:103-104 style dip
    ref = orc.strand_run(types, coeff, orc.model("default"), stop_time=200.0, rec_every=50)
    sim = lq.Sim(types, 0.15, coeff_1d=coeff, precision=lq.FP64, model="default")
    mask = np.zeros(100, np.uint8)
    mask[:3] = 1
    sim.set_protocol(bcl=1000.0, s1_mask=mask, s1_start=50.0, s1_duration=1.0, s1_strength=-52.0)
    out = []
    for _ in range(len(ref["rec"])):
        sim.step(1)
        out.append(sim.get_v(as_double=True))
        sim.step(49)
    out = np.array(out)
    assert np.abs(out - ref["rec"]).max() < 1e-6


def test_checkpoint_roundtrip_and_blowup_counter(lq, orc, tmp_path):
    sh, fib = small_sheet(lq, 24)
    sim = lq.Sim(sh.types, 0.15, precision=lq.MIXED)
    sim.set_protocol(bcl=1000.0, s1_mask=sh.s1_mask, s1_duration=2.0)
    sim.step(120)
    p = str(tmp_path / "ck.bin")
    sim.checkpoint(p)
    s0 = sim.get_state()
    sim.step(80)
    a = sim.get_state()
    sim.restore(p)
    assert abs(sim.time - 120 * 0.02) < 1e-9
    np.testing.assert_array_equal(sim.get_state(), s0)
    sim.step(80)
    np.testing.assert_array_equal(sim.get_state(), a)
    assert sim.check() == 0
    # a NaN planted in the host state is reported by the device counter
    bad = sim.get_state()
    bad[5, 0] = np.nan
    sim.set_state(bad)
    sim.step(1)
    assert sim.check() >= 1


def test_occupancy_variants_are_bitwise_identical(lq):
    """The autotuner's kernel variants differ only in register allocation."""
    v = small_ventricle(lq)
    states = []
    for variant in (2, 3, 4):
        sim = lq.Sim(v.types, 0.2, fibre=v.fibre, precision=lq.MIXED, model="default")
        sim.set_protocol(bcl=800.0, s1_mask=v.s1_mask, s1_duration=2.0)
        assert sim.tune(variant)[0] == variant
        sim.step(150)
        states.append(sim.get_state())
    assert np.array_equal(states[0], states[1]) and np.array_equal(states[0], states[2])
    sim.tune(-1)              # the autotuner runs and picks one of them
    assert sim.tune(-1)[0] in (2, 3, 4)


@pytest.mark.gpu
def test_async_v_readback_matches_sync(lq):
    """lqt_sim_get_v_async: the copies overlap later steps and still deliver
    the V of the step they were issued after."""
    import torch
    sh = lq.geometry.sheet(60, 60, s1_cols=3)
    sim = lq.Sim(sh.types, 0.15, precision=lq.MIXED, model="lqt1")
    sim.set_protocol(bcl=1000.0, s1_mask=sh.s1_mask, s1_start=0.0, s1_duration=2.0, s1_strength=-52.0)
    bufs = [torch.empty(sim.n, dtype=torch.float32, pin_memory=True).numpy() for _ in range(6)]
    ref = []
    for i in range(6):
        sim.step(40)
        ref.append(sim.get_v())
        sim.get_v_async(bufs[i])
    sim.wait_v()
    for i in range(6):
        np.testing.assert_array_equal(bufs[i], ref[i])
    # double precision buffers too
    b64 = np.zeros(sim.n)
    sim.step(7)
    assert sim.get_v_async(b64) == 6
    sim.wait_v()
    np.testing.assert_array_equal(b64, sim.get_v(as_double=True))
    # a copy not issued yet is refused
    with pytest.raises(lq.LqtError):
        sim.wait_v(7)


@pytest.mark.gpu
def test_async_v_readback_ring_waits_per_copy(lq):
    """More copies than the 16 device slots and the 64 kept completion
    events, with a host ring of 5 buffers: before a buffer is reused the host
    waits for the copy that last filled it (lqt_sim_wait_v_upto), which then
    holds the V of its step."""
    import torch
    sh = lq.geometry.sheet(50, 40, s1_cols=3)
    sim = lq.Sim(sh.types, 0.15, precision=lq.MIXED, model="lqt1")
    sim.set_protocol(bcl=1000.0, s1_mask=sh.s1_mask, s1_start=0.0, s1_duration=2.0, s1_strength=-52.0)
    ring = 5
    bufs = [torch.empty(sim.n, dtype=torch.float32, pin_memory=True).numpy() for _ in range(ring)]
    ref, checked = [], 0
    for i in range(90):
        sim.step(3)
        ref.append(sim.get_v())
        if i >= ring:
            sim.wait_v(i - ring)
            np.testing.assert_array_equal(bufs[i % ring], ref[i - ring])
            checked += 1
        assert sim.get_v_async(bufs[i % ring]) == i
    sim.wait_v(89)
    for i in range(85, 90):
        np.testing.assert_array_equal(bufs[i % ring], ref[i])
    sim.wait_v(3)                       # long complete: returns at once
    assert checked == 85


def test_async_steps_match_synchronous_steps(lq):
    """lqt_sim_step_async: single steps enqueued without waiting, each with a
    V read-back into a ring of pinned buffers, give the same bits as
    lqt_sim_step over the same steps; every read-back holds the V of its
    step.  The surrogate is attached, so macro steps and substeps are among
    the enqueued work."""
    import torch
    from lqt1_gb300 import surrogate as S
    net = S.load()
    v = lq.geometry.ventricle(nx=44, ny=44, nz=50, dx=0.2, a_out=4.0, c_out=8.0, wall=2.0, z_base=9.0,
                              island_radius=1.5, stim_radius=1.2)
    m = lq.model("baseline", gks_scale=0.5, pca_scale=2.0, gks_iso_scale=1.5)

    def make():
        sim = lq.Sim(v.types, 0.2, fibre=v.fibre, precision=lq.MIXED, model=m)
        sim.set_protocol(bcl=800.0, s1_mask=v.s1_mask, s1_start=0.0, s1_duration=2.0, s1_strength=-52.0)
        sim.set_surrogate(net)
        sim.tune(4)
        sim.substep_variant(5)
        return sim
    a, b = make(), make()
    a.step(5)
    b.step(5)
    K, ring = 120, 16
    bufs = [torch.empty(a.n, dtype=torch.float32, pin_memory=True).numpy() for _ in range(ring)]
    ref = []
    for i in range(K):
        a.step_async(1)
        if i >= ring:
            a.wait_v(i - ring)          # the copy that last filled this buffer
            np.testing.assert_array_equal(bufs[i % ring], ref[i - ring])
        assert a.get_v_async(bufs[i % ring]) == i
        b.step(1)
        ref.append(b.get_v())
    a.sync()
    a.wait_v()
    np.testing.assert_array_equal(a.get_state(), b.get_state())
    assert a.surrogate_stats() == b.surrogate_stats()
    assert a.time == b.time
    a.close()
    b.close()
