"""The tissue numbering and mirror-boundary map built on the GPU
(lqt_geom_mirror_map_gpu, the builder lqt_sim_create uses) against the host
builder, which the CPU tests pin to the oracle's restatement of
GPU3D.cu:1487-1604 / new_11.cu:1535-1640: bit-identical numbering, boundary
list and mirror sources on random 2D/3D shapes (tissue on the grid faces
included), a small ventricle and the full 320 x 320 x 420 workload grid."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    import lqt1_gb300 as lq
    lq.lib()
    from lqt1_gb300 import geometry
    return geometry


def _same(G, types):
    t0 = time.perf_counter()
    host = G.mirror_map(types)
    t1 = time.perf_counter()
    dev = G.mirror_map(types, gpu=True)
    t2 = time.perf_counter()
    for a, b in zip(host, dev):
        np.testing.assert_array_equal(a, b)
    return len(host[1]), t1 - t0, t2 - t1


@pytest.mark.parametrize("shape", [(30, 28), (64, 3), (16, 18, 20), (40, 33, 27)])
def test_random_shapes(G, shape):
    rng = np.random.default_rng(sum(shape))
    for fill in (0.3, 0.6, 0.9):
        g = np.where(rng.random(shape) < fill, rng.integers(2, 5, shape), 255).astype(np.uint8)
        nb, _, _ = _same(G, g)           # tissue on the faces too: the map is still defined
        assert nb > 0


def test_sheet_and_small_ventricle(G):
    _same(G, G.sheet(50, 40).types)
    v = G.ventricle(nx=44, ny=44, nz=50, dx=0.2, a_out=4.0, c_out=8.0, wall=2.0, z_base=9.0, island_radius=1.5,
                    stim_radius=1.0)
    nb, _, _ = _same(G, v.types)
    assert nb > 1000


def test_full_workload_grid(G):
    v = G.ventricle()
    nb, t_host, t_gpu = _same(G, v.types)
    assert nb > 100_000
    print(f"mirror map of 320x320x420: {nb} boundary voxels; host {t_host:.2f} s, GPU {t_gpu:.2f} s")
