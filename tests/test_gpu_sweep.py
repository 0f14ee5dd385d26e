"""GPU parity of the batched sweep (uneven single cells and strands with their
own parameters, one persistent graph-captured launch) against FP64
single-instance oracle runs with the same AP detector."""
import concurrent.futures as cf

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lq():
    import lqt1_gb300 as lq
    lq.lib()
    return lq


def oracle_instance(orc, spec, m, dt=0.02, beats=4):
    mo = orc.model(dict(dss_shift=m.dss_shift, fss_shift=m.fss_shift, pca_scale=m.pca_scale, gks_scale=m.gks_scale,
                        gks_iso_scale=m.gks_iso_scale, suprep_dose=m.suprep_dose))
    n = len(spec.types)
    return orc.strand_detect(spec.types, np.full(n, 0.154), mo, dx=spec.dx, dt=dt, bcl=spec.bcl,
                             stim_start=spec.s1_start, stim_dur=spec.s1_duration, stim_strength=spec.s1_strength,
                             n_stim=spec.n_stim, s1_beats=spec.s1_beats, stop_time=spec.t_stop, max_beats=beats)


def test_sweep_mixed_vs_fp64_oracle(lq, orc):
    insts, models, _ = lq.batch.sweep(n=40, seed=5, beats=2, len_range=(50, 90), bcl_range=(400.0, 900.0))
    b = lq.Batch(insts, models, precision=lq.MIXED, max_beats=4)
    ms = b.run()
    assert ms > 0 and b.num_bad() == 0
    got = b.detect()
    with cf.ThreadPoolExecutor(8) as ex:
        refs = list(ex.map(lambda sm: oracle_instance(orc, *sm), zip(insts, models)))
    off = b.offsets
    n_apd = 0
    for i, (spec, ref) in enumerate(zip(insts, refs)):
        sl = slice(off[i], off[i + 1])
        ta, ap = got["t_act"][sl, :2], got["apd90"][sl, :2]
        rta, rap = ref["t_act"][:, :2], ref["apd90"][:, :2]
        assert np.array_equal(ta >= 0, rta >= 0), i
        both = (ta >= 0) & (rta >= 0)
        assert np.abs(ta[both] - rta[both]).max() <= 0.1 + 1e-3, i
        both = (ap >= 0) & (rap >= 0)
        assert np.array_equal(ap >= 0, rap >= 0), i
        if both.any():
            assert np.abs(ap[both] - rap[both]).max() <= 1.0, (i, np.abs(ap[both] - rap[both]).max())
            n_apd += both.sum()
        assert np.array_equal(got["ead"][sl], ref["ead"]), i
    assert n_apd > 1000


def test_sweep_autotune_and_rerun_is_deterministic(lq):
    insts, models, _ = lq.batch.sweep(n=64, seed=9, beats=1, len_range=(50, 300), bcl_range=(400.0, 600.0))
    b = lq.Batch(insts, models, precision=lq.MIXED, max_beats=2)
    cfg = b.config()
    assert cfg["threads"] >= 300 and cfg["nitems"] >= 1
    s0 = b.get_state()
    b.run()
    a = b.get_state()
    b.set_state(s0)
    b.run()
    assert np.array_equal(a, b.get_state())


def test_sweep_at_stated_size_vs_fp64_oracle(lq, orc):
    """The batched sweep as stated (4096 instances, single cells and strands of
    50-400 cells, BCL 400-2000 ms, 20 beats), checked on a seeded sub-sample
    against FP64 oracle instances: 24 single cells (the 12 most EAD-prone by
    IKs loss x ICaL gain and 12 spread over the BCL range, the longest
    included) and two strands that stretch the ranges: 394 cells at BCL
    424 ms, and 66 cells at BCL 1997 ms (20 beats of a 400-cell strand at a
    2 s BCL would take the host oracle many minutes).  The sub-sample runs
    as its own batch (an instance's arithmetic does not depend on its
    neighbours); per cell and beat: activation within 0.1 ms, APD90 within
    1 ms, the same EAD flag."""
    insts, models, params = lq.batch.sweep(n=4096, seed=2024, beats=20)
    singles = [i for i, p in enumerate(params) if p["single"]]
    prone = sorted(singles, key=lambda i: -params[i]["mut"] * params[i]["ical"] / params[i]["iks"])[:12]
    by_bcl = sorted(singles, key=lambda i: params[i]["bcl"])
    spread = [by_bcl[int(round(k * (len(by_bcl) - 1) / 11))] for k in range(12)]
    pick = sorted(set(prone + spread)) + [3931, 2181]
    assert params[3931]["ncells"] == 394 and params[2181]["ncells"] == 66 and params[2181]["bcl"] > 1995.0
    assert max(params[i]["bcl"] for i in pick) > 1995.0
    sub = [insts[i] for i in pick]
    sub_models = [models[i] for i in pick]
    for j, x in enumerate(sub):
        x.model = j
    b = lq.Batch(sub, sub_models, precision=lq.MIXED, max_beats=21)
    b.run()
    assert b.num_bad() == 0
    got = b.detect()
    with cf.ThreadPoolExecutor(4) as ex:
        refs = list(ex.map(lambda sm: oracle_instance(orc, *sm, beats=21), zip(sub, sub_models)))
    off = b.offsets
    n_apd = 0
    for i, (spec, ref) in enumerate(zip(sub, refs)):
        sl = slice(off[i], off[i + 1])
        ta, ap = got["t_act"][sl], got["apd90"][sl]
        rta, rap = ref["t_act"], ref["apd90"]
        assert np.array_equal(ta >= 0, rta >= 0), pick[i]
        both = (ta >= 0) & (rta >= 0)
        assert np.abs(ta[both] - rta[both]).max() <= 0.1 + 1e-3, pick[i]
        assert np.array_equal(ap >= 0, rap >= 0), pick[i]
        both = (ap >= 0) & (rap >= 0)
        assert np.abs(ap[both] - rap[both]).max() <= 1.0, (pick[i], np.abs(ap[both] - rap[both]).max())
        n_apd += both.sum()
        assert np.array_equal(got["ead"][sl], ref["ead"]), pick[i]
    assert n_apd > 0.8 * 20 * sum(len(x.types) for x in sub)
