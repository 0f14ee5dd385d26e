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
