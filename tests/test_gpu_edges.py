"""Edge cases of the path on the GPU: degenerate grids and strands, empty and
maximum-size batch instances, the surrogate on a 1D strand and where nothing
is eligible, lattice sampling with a stride beyond the grid."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lq():
    import lqt1_gb300 as lq
    lq.lib()
    return lq


@pytest.mark.parametrize("shape", [(3, 3), (3, 3, 3), (5, 4, 3)])
def test_single_tissue_voxel_grid_fp64_vs_oracle(lq, orc, shape):
    """One tissue voxel surrounded by empty voxels: its mirror ghosts hold
    its own V, so diffusion vanishes and it behaves as a single cell."""
    types = np.full(shape, 255, np.uint8)
    c = tuple(s // 2 for s in shape)
    types[c] = lq.MCELL
    s1 = np.zeros(shape, np.uint8)
    s1[c] = 1
    sim = lq.Sim(types, 0.2, precision=lq.FP64, model="default")
    sim.set_protocol(bcl=1000.0, s1_mask=s1, s1_start=0.0, s1_duration=2.0, s1_strength=-52.0)
    assert sim.n == 1
    sim.step(400)
    og = orc.Grid(types, 0.2)
    st = orc.initial_state(-87.5, og.n)
    t = 0.0
    for _ in range(400):
        og.step(st, orc.model("default"), 0.02,
                np.array([-52.0 if orc.in_window(t, 1000.0, 0.0, 2.0) else 0.0]))
        t += 0.02
    got = sim.get_state()
    assert abs(got[0, 0] - st[0, 0]) < 1e-3
    np.testing.assert_allclose(got[:, 1:], st[:, 1:], rtol=1e-4, atol=1e-7)
    assert got[0, 0] > 0.0                             # it fired


@pytest.mark.parametrize("n", [1, 2])
def test_tiny_strands_fp64_vs_oracle(lq, orc, n):
    types = np.array([lq.ENDO, lq.EPI][:n], np.uint8)
    coeff = np.full(n, 0.154)
    ref = orc.strand_run(types, coeff, orc.model("default"), stop_time=400.0, rec_every=0, n_stim=1)
    sim = lq.Sim(types, 0.15, coeff_1d=coeff, precision=lq.FP64, model="default")
    mask = np.zeros(n, np.uint8)
    mask[0] = 1
    sim.set_protocol(bcl=1000.0, s1_mask=mask, s1_start=50.0, s1_duration=1.0, s1_strength=-52.0)
    t, nsteps = 0.0, 0
    while t <= 400.0:                 # the oracle's loop: steps while time <= stop (OneD.cc:317)
        t += 0.02
        nsteps += 1
    sim.step(nsteps)
    got = sim.get_state()
    assert np.abs(got[:, 0] - ref["final"][:, 0]).max() < 1e-3
    np.testing.assert_allclose(got[:, 1:], ref["final"][:, 1:], rtol=1e-4, atol=1e-7)


def test_batch_shortest_and_maximum_instances(lq, orc):
    """A batch mixing an instance that runs one step (t_stop = 0: steps while
    time <= t_stop), a single cell, and a strand of the maximum length (512
    cells)."""
    m = lq.model("default")
    long_types = np.array([lq.ENDO] * 128 + [lq.MCELL] * 184 + [lq.EPI] * 200, np.uint8)
    insts = [lq.InstanceSpec(types=np.array([lq.EPI], np.uint8), t_stop=0.0, n_stim=1),
             lq.InstanceSpec(types=np.array([lq.MCELL], np.uint8), t_stop=300.0, n_stim=1),
             lq.InstanceSpec(types=long_types, t_stop=300.0, n_stim=3)]
    b = lq.Batch(insts, [m], precision=lq.FP64, max_beats=2)
    b.run()
    st = b.get_state()
    one = orc.cells_update(orc.initial_state(-87.5), [orc.EPI], orc.model("default"), nsteps=1)[0]
    np.testing.assert_allclose(st[0], one, rtol=1e-12, atol=1e-15)   # exactly one step ran
    ref = orc.strand_run(long_types, np.full(512, 0.154), orc.model("default"), stop_time=300.0, rec_every=0)
    assert np.abs(st[2:, 0] - ref["final"][:, 0]).max() < 1e-3
    np.testing.assert_allclose(st[2:, 1:], ref["final"][:, 1:], rtol=1e-4, atol=1e-7)
    det = b.detect()
    assert det["t_act"][2 + 511, 0] > det["t_act"][2, 0] > 0        # the wave crossed the strand
    b.close()
    with pytest.raises(lq.LqtError):                                 # beyond the CTA width
        lq.Batch([lq.InstanceSpec(types=np.zeros(513, np.uint8) + lq.ENDO)], [m])


def test_surrogate_on_a_strand_and_with_nothing_eligible(lq):
    """The macro step and the V-only substep on a 1D strand (dim 1 paths),
    against the plain mixed strand; and a run whose voxels are never offered
    (a stimulus every cycle keeps the cells in upstroke / stimulated)."""
    from lqt1_gb300 import surrogate as S
    net = S.load()
    types = lq.oned_types()
    mask = np.zeros(100, np.uint8)
    mask[:3] = 1
    model = lq.model("baseline", gks_scale=0.5, pca_scale=1.5, gks_iso_scale=1.2)
    out = {}
    for sur in (False, True):
        sim = lq.Sim(types, 0.15, precision=lq.MIXED, model=model)
        sim.set_protocol(bcl=1000.0, s1_mask=mask, s1_start=50.0, s1_duration=1.0, s1_strength=-52.0)
        if sur:
            sim.set_surrogate(net)
        sim.step(25000)
        out[sur] = (sim.detect(), sim.surrogate_stats() if sur else None, sim.check())
        sim.close()
    dp, _, badp = out[False]
    ds, st, bads = out[True]
    assert badp == 0 and bads == 0
    assert st["accepted"] > 0.5 * st["macro_steps"] * 100
    both = (dp["apd90"] > 0) & (ds["apd90"] > 0)
    assert both.all()
    assert np.abs(dp["apd90"] - ds["apd90"]).max() < 1.0
    assert np.abs(dp["t_act"] - ds["t_act"]).max() <= 0.1 + 1e-4
    # nothing eligible: every voxel stimulated with a 1000 ms window every cycle
    sh = lq.geometry.sheet(10, 10, s1_cols=1)
    sim = lq.Sim(sh.types, 0.15, precision=lq.MIXED, model=model)
    sim.set_protocol(bcl=5.0, s1_mask=(sh.types != 255).astype(np.uint8), s1_start=0.0, s1_duration=5.0,
                     s1_strength=-1.0)
    sim.set_surrogate(net)
    sim.step(100)
    st = sim.surrogate_stats()
    assert st["macro_steps"] == 100 // net.nsub and st["offered"] == 0 and st["accepted"] == 0
    assert sim.check() == 0
    # models outside the network's inputs (gate shifts, SUPREP) are refused
    sim2 = lq.Sim(sh.types, 0.15, precision=lq.MIXED, model="default")
    with pytest.raises(lq.LqtError):
        sim2.set_surrogate(net)


def test_sampling_stride_beyond_the_grid(lq):
    sh = lq.geometry.sheet(8, 6, s1_cols=1)
    sim = lq.Sim(sh.types, 0.15, precision=lq.MIXED, model="lqt1")
    smp = sim.sample_v(50)
    assert smp.shape == (1,) and smp[0] == -100.0                    # (0, 0) is an empty corner
    full = sim.sample_v(1)
    assert full.shape == (sh.types.size,)
    assert (full[sh.types.T.reshape(-1) != 255] == -87.5).all()
