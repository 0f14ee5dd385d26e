"""Oracle restatement vs the reference's own TPORd::update() built from its
sources by oracle/build_ref.sh (x86 container only; skipped elsewhere)."""
import numpy as np
import pytest


@pytest.mark.parametrize("variant", ["default", "baseline", "lqt1", "lqt1half", "suprep"])
def test_random_states_bitwise(orc, variant):
    if not orc.ref_available(variant):
        pytest.skip("reference build (oracle/_ref) not present on this host")
    rng = np.random.default_rng(7)
    n = 4096
    s0 = orc.random_states(n, seed=11)
    types = rng.integers(0, 5, n).astype(np.uint8)
    ist = np.where(rng.random(n) < 0.2, -52.0, 0.0)
    dg = rng.normal(0, 5, n)
    a = orc.cells_update(s0.copy(), types, orc.model(variant), ist=ist, dvgap=dg, nsteps=100)
    b = orc.ref_update(s0.copy(), types, variant, ist=ist, dvgap=dg, nsteps=100)
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


@pytest.mark.parametrize("variant", ["default", "lqt1half"])
def test_current_getters_bitwise(orc, variant):
    """getINa / getICaL / getIKr / getIKs / getIK1 / getAbsDvdt of the last
    update (SingleCell/TPORd.cc:358-376) against the oracle's currents."""
    if not orc.ref_available(variant):
        pytest.skip("reference build (oracle/_ref) not present on this host")
    rng = np.random.default_rng(8)
    n = 2048
    s0 = orc.random_states(n, seed=12)
    types = rng.integers(0, 5, n).astype(np.uint8)
    ist = np.where(rng.random(n) < 0.2, -52.0, 0.0)
    dg = rng.normal(0, 5, n)
    sa, sb = s0.copy(), s0.copy()
    a = orc.cells_currents(sa, types, orc.model(variant), ist=ist, dvgap=dg, nsteps=7)
    b = orc.ref_currents(sb, types, variant, ist=ist, dvgap=dg, nsteps=7)
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
    assert np.array_equal(sa.view(np.uint64), sb.view(np.uint64))
    # getAbsDvdt is the magnitude as a double (no truncation to an integer)
    assert (b[:, 5] != np.floor(b[:, 5])).any()


def test_text_state_io_matches_reference(orc, lq_lib, tmp_path):
    """lqt_state_write_text writes the bytes of the reference's
    outputAllStates, cell after cell; lqt_state_read_text reads what the
    reference's readinAllStates reads, from the reference's own file."""
    if not orc.ref_available("default"):
        pytest.skip("reference build (oracle/_ref) not present on this host")
    from lqt1_gb300 import _native as N
    s = orc.random_states(5, seed=13)
    s[2, 7] = -0.00000000004          # rounds to -0.0000000000 in "%4.10f"
    s[3, 0] = 1234.56789012345
    ref_path, our_path = str(tmp_path / "ref.dat"), str(tmp_path / "ours.dat")
    orc.ref_write_states(s, ref_path)
    with N.CFile(our_path, "w") as f:
        assert lq_lib.lqt_state_write_text(s.ctypes.data, len(s), f.ptr) == 0
    assert open(ref_path, "rb").read() == open(our_path, "rb").read()
    back = np.zeros_like(s)
    with N.CFile(ref_path, "r") as f:
        assert lq_lib.lqt_state_read_text(back.ctypes.data, len(s), f.ptr) == 0
    want = orc.ref_read_states(len(s), ref_path)
    assert np.array_equal(back.view(np.uint64), want.view(np.uint64))
    # a short file is an I/O error
    with N.CFile(ref_path, "r") as f:
        assert lq_lib.lqt_state_read_text(back.ctypes.data, len(s) + 1, f.ptr) == N.ERR_IO
    assert b"missing" in lq_lib.lqt_last_error()
