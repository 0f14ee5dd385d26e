"""GPU parity: the Cell interface (lqt_cells_*) against the CPU oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lq():
    import lqt1_gb300 as lq
    lq.lib()
    return lq


def _random(orc, n, seed):
    rng = np.random.default_rng(seed)
    s = orc.random_states(n, seed=seed)
    types = rng.integers(0, 5, n).astype(np.uint8)
    ist = np.where(rng.random(n) < 0.2, -52.0, 0.0)
    dg = rng.normal(0, 5, n)
    return s, types, ist, dg


@pytest.mark.parametrize("preset", ["default", "lqt1", "gpu3d"])
def test_fp64_one_step_matches_oracle(lq, orc, preset):
    """FP64 form, one TPORd::update() per cell: every state within 1e-9
    relative (CUDA vs glibc exp/log differ in the last bits only)."""
    n = 4096
    s, types, ist, dg = _random(orc, n, 3)
    ref = orc.cells_update(s.copy(), types, orc.model(preset), ist=ist, dvgap=dg, nsteps=1)
    c = lq.TPORdCells(types, precision=lq.FP64, model=preset)
    c.set_state(s)
    c.set_istim(ist)
    c.set_dvgap_dt(dg)
    c.update(1)
    got = c.get_state()
    np.testing.assert_allclose(got, ref, rtol=1e-9, atol=1e-12)


def test_fp64_many_steps_matches_oracle(lq, orc):
    n = 2048
    s, types, ist, dg = _random(orc, n, 5)
    ref = orc.cells_update(s.copy(), types, orc.model("default"), ist=ist, dvgap=dg, nsteps=200)
    c = lq.TPORdCells(types, precision=lq.FP64, model="default")
    c.set_state(s)
    c.set_istim(ist)
    c.set_dvgap_dt(dg)
    c.update(200)
    got = c.get_state()
    assert np.abs(got[:, 0] - ref[:, 0]).max() < 1e-6          # V, mV
    np.testing.assert_allclose(got, ref, rtol=1e-6, atol=1e-9)


def test_mixed_one_step_close_to_oracle(lq, orc):
    """Mixed form (FP32 gates/currents, FP64 concentrations), one step."""
    n = 4096
    s, types, ist, dg = _random(orc, n, 9)
    ref = orc.cells_update(s.copy(), types, orc.model("default"), ist=ist, dvgap=dg, nsteps=1)
    c = lq.TPORdCells(types, precision=lq.MIXED, model="default")
    c.set_state(s)
    c.set_istim(ist)
    c.set_dvgap_dt(dg)
    c.update(1)
    got = c.get_state()
    assert np.abs(got[:, 0] - ref[:, 0]).max() < 2e-3           # mV
    assert np.abs(got[:, 9:37] - ref[:, 9:37]).max() < 1e-4     # gates
    np.testing.assert_allclose(got[:, 1:9], ref[:, 1:9], rtol=1e-5)


def test_state_roundtrip_and_dump(lq, orc, tmp_path):
    s, types, _, _ = _random(orc, 64, 1)
    for prec in (lq.FP64, lq.MIXED):
        c = lq.TPORdCells(types, precision=prec)
        c.set_state(s)
        got = c.get_state()
        if prec == lq.FP64:
            assert np.array_equal(got, s)
        else:
            np.testing.assert_allclose(got, s, rtol=1e-7)
        c.output_all_states(str(tmp_path / "st.dat"), 3)
        lines = open(tmp_path / "st.dat").read().split()
        assert len(lines) == 40
        np.testing.assert_allclose(np.array(lines, float), got[3], rtol=0, atol=5.1e-11)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_current_getters_match_oracle(lq, orc, prec):
    """getINa / getICaL / getIKr / getIKs / getIK1 / getAbsDvdt of the last
    update (SingleCell/TPORd.cc:358-376) after 7 updates, against the oracle
    (itself bit-identical to the reference's getters): FP64 within the last
    bits of the exp/log differences; mixed within 1e-3 of each current's
    scale (INa's scale is its upstroke peak)."""
    n = 4096
    s, types, ist, dg = _random(orc, n, 17)
    ref = orc.cells_currents(s.copy(), types, orc.model("default"), ist=ist, dvgap=dg, nsteps=7)
    c = lq.TPORdCells(types, precision=lq.FP64 if prec == "fp64" else lq.MIXED, model="default")
    assert not c.get_currents().any()               # nothing before the first update
    c.set_state(s)
    c.set_istim(ist)
    c.set_dvgap_dt(dg)
    c.update(7)
    got = c.get_currents()
    scale = np.abs(ref).max(axis=0)
    if prec == "fp64":
        np.testing.assert_allclose(got, ref, rtol=1e-8, atol=1e-10 * scale.max())
    else:
        assert (np.abs(got - ref).max(axis=0) <= 1e-3 * scale).all(), np.abs(got - ref).max(axis=0) / scale
    assert (got[:, 5] >= 0).all()
    np.testing.assert_array_equal(got[:, 5], np.abs(c.get_dvdt()))


def test_text_states_through_the_c_abi(lq, orc, tmp_path):
    """outputAllStates / readinAllStates through lqt_cells_output_states and
    lqt_cells_readin_states on one stream: two ranges of cells written one
    after the other give the oracle's "%4.10f" lines, and reading them back
    into other cells restores those states to the printed precision; a short
    file leaves every cell unchanged."""
    from lqt1_gb300 import _native as N
    s, types, _, _ = _random(orc, 32, 5)
    c = lq.TPORdCells(types, precision=lq.FP64)
    c.set_state(s)
    path = str(tmp_path / "states.dat")
    L = lq.lib()
    with N.CFile(path, "w") as f:
        assert L.lqt_cells_output_states(c._h, 2, 3, f.ptr) == 0
        assert L.lqt_cells_output_states(c._h, 20, 1, f.ptr) == 0
    want = "".join("%4.10f\n" % x for x in np.concatenate([s[2:5].ravel(), s[20]]))
    assert open(path).read() == want
    with N.CFile(path, "r") as f:
        assert L.lqt_cells_readin_states(c._h, 10, 4, f.ptr) == 0
    got = c.get_state()
    np.testing.assert_allclose(got[10:14], np.concatenate([s[2:5], s[20:21]]), rtol=0, atol=5.1e-11)
    np.testing.assert_array_equal(got[:10], s[:10])
    np.testing.assert_array_equal(got[14:], s[14:])
    with N.CFile(path, "r") as f:
        assert L.lqt_cells_readin_states(c._h, 0, 5, f.ptr) == N.ERR_IO
    np.testing.assert_array_equal(c.get_state(), got)
    with N.CFile(path, "r") as f:
        assert L.lqt_cells_readin_states(c._h, 30, 4, f.ptr) == N.ERR_INVALID
