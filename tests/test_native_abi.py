"""CPU checks of the C ABI: the library loads, exports every function that
include/lqt.h declares, and its host-only functions agree with the oracle."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lq():
    import lqt1_gb300 as lq
    lq.lib()
    return lq


def header_functions():
    src = open(os.path.join(ROOT, "include", "lqt.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(lqt_[a-z0-9_]+)\s*\(", src)))


def test_exports_every_declared_symbol(lq):
    names = header_functions()
    assert len(names) > 40
    missing = [n for n in names if not hasattr(lq.lib(), n)]
    assert not missing, missing


def test_presets_match_reference_builds(lq):
    m = lq.model("default")          # CON + ISO1 (SingleCell/TPORd.cc:33,35)
    assert (m.dss_shift, m.fss_shift, m.pca_scale, m.gks_scale, m.gks_iso_scale, m.suprep_dose) == (12, 8, 1.6, 1, 3.2, 0)
    m = lq.model("gpu3d")            # LQT1 + ISO1 + SUPREP (GPU3D.cu:18-22)
    assert (m.pca_scale, m.gks_scale, m.gks_iso_scale, m.suprep_dose) == (4.0, 0.05, 3.2, 100.0)
    with pytest.raises(lq.LqtError):
        lq._native.check(lq.lib().lqt_model_preset(99, C.byref(lq.Model())), "lqt_model_preset")


def test_initial_state_matches_oracle(lq, orc):
    assert np.array_equal(lq.initial_state(-86.2), orc.initial_state(-86.2)[0])


def test_invalid_arguments_are_rejected_without_a_gpu(lq):
    h = C.c_void_p()
    rc = lq.lib().lqt_cells_create(0, None, 1, None, 0.02, None, C.byref(h))
    assert rc == 1 and b"n <= 0" in lq.lib().lqt_last_error()
    rc = lq.lib().lqt_batch_create(None, 0, None, None, None, 0, None, C.byref(h))
    assert rc == 1


def test_surrogate_arguments_are_rejected_without_a_gpu(lq):
    """Training-pair ranges with a macro length that does not divide the
    50-step graph span, or a non-zero reserved field, are refused before any
    device work; so are NULL handles of the surrogate and tuning calls."""
    from lqt1_gb300 import surrogate as S
    L = S._bind_sur()

    def ranges(nsub, reserved=0, prob=0.01):
        return S.SurRanges((C.c_double * 2)(0.05, 1.0), (C.c_double * 2)(1.0, 2.2), (C.c_double * 2)(1.0, 2.0),
                           (C.c_double * 2)(400.0, 2000.0), 0, 2, 0.02, 2.0, prob, 0.3, nsub, reserved)
    n = C.c_int64()
    for bad in (ranges(7), ranges(51), ranges(-5), ranges(10, reserved=1), ranges(10, prob=0.0)):
        rc = L.lqt_sur_datagen(16, 1, C.byref(bad), C.c_void_p(16), C.c_void_p(16), 100, C.byref(n), None)
        assert rc == lq._native.ERR_INVALID, lq.lib().lqt_last_error()
    rc = L.lqt_sur_datagen(16, 1, None, C.c_void_p(16), C.c_void_p(16), 100, C.byref(n), None)
    assert rc == lq._native.ERR_INVALID
    lib = lq.lib()
    lib.lqt_sim_substep_variant.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]
    lib.lqt_sim_set_wait_test.argtypes = [C.c_void_p, C.c_int32, C.c_uint32]
    lib.lqt_sim_surrogate_rejections.argtypes = [C.c_void_p, C.c_void_p]
    assert lib.lqt_sim_substep_variant(None, 105, None, None) == lq._native.ERR_INVALID
    assert lib.lqt_sim_set_wait_test(None, 1, 16) == lq._native.ERR_INVALID
    assert lib.lqt_sim_surrogate_rejections(None, None) == lq._native.ERR_INVALID
    assert lib.lqt_sim_step_async(None, 1) == lq._native.ERR_INVALID
    assert lib.lqt_sim_sync(None) == lq._native.ERR_INVALID
    lib.lqt_sim_wait_v_upto.argtypes = [C.c_void_p, C.c_int64]
    assert lib.lqt_sim_wait_v_upto(None, 0) == lq._native.ERR_INVALID


def _compare_maps(lq, orc, grid):
    from lqt1_gb300 import geometry as G
    tof, dst, src = G.mirror_map(grid)
    og = orc.Grid(grid, 0.2)
    ot = og.tissue_of
    assert np.array_equal(tof[tof >= 0], ot[ot >= 0])
    bmask = (ot < 0) & (ot != np.iinfo(np.int32).min)
    assert np.array_equal(np.nonzero(bmask)[0], np.sort(dst))
    # oracle stores -(tissue index + 1) of the source
    src_t = -ot[dst] - 1
    assert np.array_equal(og.tissue_cell[src_t], src)


def test_mirror_map_matches_oracle_random_shapes(lq, orc):
    rng = np.random.default_rng(4)
    for shape in [(30, 28), (16, 18, 20)]:
        g = np.full(shape, 255, np.uint8)
        inner = tuple(slice(1, s - 1) for s in shape)
        blob = rng.random(tuple(s - 2 for s in shape)) < 0.6
        g[inner] = np.where(blob, 3, 255)
        _compare_maps(lq, orc, g)


def test_mirror_map_matches_oracle_ventricle(lq, orc):
    from lqt1_gb300 import geometry as G
    v = G.ventricle(nx=44, ny=44, nz=50, dx=0.2, a_out=4.0, c_out=8.0, wall=2.0, z_base=9.0, island_radius=1.5,
                    stim_radius=1.0)
    assert (v.types != 255).sum() > 10000
    _compare_maps(lq, orc, v.types)


def test_full_ventricle_geometry(lq):
    from lqt1_gb300 import geometry as G
    v = G.ventricle()
    n = int((v.types != 255).sum())
    assert 6.5e6 < n < 7.5e6, n            # about 7M tissue voxels
    t = v.types[v.types != 255]
    assert set(np.unique(t)) == {2, 3, 4}
    f = v.fibre[v.types != 255]
    assert np.allclose(np.linalg.norm(f, axis=1), 1, atol=1e-5)
    # tissue stays off the grid faces
    for ax in range(3):
        assert (np.take(v.types, 0, axis=ax) == 255).all() and (np.take(v.types, -1, axis=ax) == 255).all()
