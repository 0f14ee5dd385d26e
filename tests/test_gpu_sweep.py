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


def oracle_instance(orc, spec, m, dt=0.02):
    mo = orc.model(dict(dss_shift=m.dss_shift, fss_shift=m.fss_shift, pca_scale=m.pca_scale, gks_scale=m.gks_scale,
                        gks_iso_scale=m.gks_iso_scale, suprep_dose=m.suprep_dose))
    n = len(spec.types)
    return orc.strand_detect(spec.types, np.full(n, 0.154), mo, dx=spec.dx, dt=dt, bcl=spec.bcl,
                             stim_start=spec.s1_start, stim_dur=spec.s1_duration, stim_strength=spec.s1_strength,
                             n_stim=spec.n_stim, s1_beats=spec.s1_beats, stop_time=spec.t_stop, max_beats=4)


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
