"""Output files in the reference drivers' formats, written by the C ABI and
compared byte for byte with a restatement of the reference's loops
(oracle/io_ref.py).  Host code only: runs without a GPU."""
import numpy as np
import pytest

from oracle import io_ref


@pytest.fixture(scope="module")
def lq():
    import lqt1_gb300 as lq
    lq.lib()
    return lq


def lattice(v, tissue, stride):
    """The sampled values in the writer's order (what lqt_sim_sample_v returns)."""
    if v.ndim == 2:
        v, tissue = v[:, :, None], tissue[:, :, None]
    s = v[::stride, ::stride, ::stride]
    t = tissue[::stride, ::stride, ::stride]
    return np.where(t, s, -100.0).transpose(2, 1, 0).reshape(-1)


@pytest.mark.parametrize("shape,stride", [((12, 9, 15), 3), ((13, 10, 8), 3), ((20, 17), 1), ((7, 7, 7), 2)])
def test_vtk_matches_reference_layout(lq, tmp_path, shape, stride):
    rng = np.random.default_rng(sum(shape))
    v = rng.normal(-40, 50, shape) * 10.0 ** rng.integers(-6, 2, shape)
    tissue = rng.random(shape) < 0.7
    p = tmp_path / "ap_0.vtk"
    lq.protocols.write_vtk(str(p), lattice(v, tissue, stride), shape, stride)
    assert p.read_text() == io_ref.vtk_text(v, tissue, stride)


def test_dat_matches_reference_format(lq, tmp_path):
    rng = np.random.default_rng(3)
    rows = np.column_stack([np.arange(7) * 0.2, rng.normal(-50, 40, (7, 100))])
    p = tmp_path / "VentOneDResults.dat"
    lq.protocols.write_oned_dat(str(p), rows[:, 0], rows[:, 1:])
    assert p.read_text() == io_ref.dat_text(rows)
    lq.protocols.write_dat(str(p), rows[:2], append=True)
    assert p.read_text() == io_ref.dat_text(rows) + io_ref.dat_text(rows[:2])


def test_writers_report_io_errors(lq, tmp_path):
    with pytest.raises(lq.LqtError):
        lq.protocols.write_dat(str(tmp_path / "no" / "such" / "dir.dat"), np.zeros((1, 2)))


def _write_geometry(path, dim, shape, rng, n):
    """A synthetic geometry file: n distinct tissue points with random codes
    0..20 and fibre vectors, points placed so that the case-study regions of
    the reference are hit."""
    pts = set()
    lines = []
    while len(lines) < n:
        p = tuple(int(rng.integers(1, s - 1)) for s in shape)
        if p in pts:
            continue
        pts.add(p)
        f = rng.normal(size=3)
        f /= np.linalg.norm(f)
        code = int(rng.integers(0, 21))
        if dim == 3:
            lines.append("%d %d %d %.6f %.6f %.6f %d" % (p + tuple(f) + (code,)))
        else:
            lines.append("%d %d %.6f %.6f %d" % (p + (f[0], f[1], code)))
    path.write_text("\n".join(lines))      # no trailing newline, as the reference requires
    return pts


@pytest.mark.parametrize("dim", [2, 3])
def test_geometry_reader_matches_reference_rules(lq, tmp_path, dim):
    rng = np.random.default_rng(dim)
    shape = (700, 500, 560) if dim == 3 else (700, 500)
    # a small dense grid would not reach the case-study regions; use a sparse set
    p = tmp_path / ("geom%d.txt" % dim)
    pts = _write_geometry(p, dim, shape, rng, 4000)
    got = lq.geometry.load_geometry(str(p), shape, case_edits=True, fibre=False)
    ref = io_ref.read_geometry_points(str(p), shape, case_edits=True)
    assert got.ntissue == len(ref) == len(pts)
    idx = tuple(np.array(list(ref.keys())).T)
    want = np.array(list(ref.values()))
    np.testing.assert_array_equal(got.types[idx], want[:, 0])
    np.testing.assert_array_equal(got.code[idx], want[:, 1])
    np.testing.assert_array_equal(got.s2_mask[idx], want[:, 2])
    assert int(np.count_nonzero(got.types != 255)) == len(ref)      # nothing else written
    # the edits changed something, and every class occurs
    raw_code = lq.geometry.load_geometry(str(p), shape, case_edits=False, fibre=False).code[idx]
    assert (raw_code != want[:, 1]).any() and want[:, 2].any()
    assert set(want[:, 0].tolist()) == {2, 3, 4}


@pytest.mark.parametrize("dim", [2, 3])
def test_geometry_reader_fibres(lq, tmp_path, dim):
    rng = np.random.default_rng(10 + dim)
    shape = (30, 25, 20) if dim == 3 else (30, 25)
    p = tmp_path / "g.txt"
    _write_geometry(p, dim, shape, rng, 300)
    got = lq.geometry.load_geometry(str(p), shape)
    ref = io_ref.read_geometry(str(p), shape)
    np.testing.assert_array_equal(got.fibre, ref[2])
    np.testing.assert_array_equal(got.types, ref[0])


def test_stimulation_reader(lq, tmp_path):
    rng = np.random.default_rng(11)
    types = np.full((40, 30, 20), 255, np.uint8)
    types[5:35, 5:25, 5:15] = 3
    lines = []
    for _ in range(500):
        x, y, z = (int(rng.integers(-2, s + 2)) for s in types.shape)
        lines.append("%d %d %d 0.1 0.2 0.3 %.4f tag" % (x, y, z, rng.uniform(0, 80)))
    p = tmp_path / "stimulationprofile.cnd"
    p.write_text("\n".join(lines) + "\n\n")
    m, on = lq.geometry.load_stimulation(str(p), types)
    mr, onr = io_ref.read_stimulation(str(p), types)
    np.testing.assert_array_equal(m, mr)
    np.testing.assert_array_equal(on, onr)
    assert 0 < m.sum() < 500
    # 2D: one layer of the profile
    t2 = types[:, :, 10].copy()
    m2, on2 = lq.geometry.load_stimulation(str(p), t2, layer=10)
    mr2, onr2 = io_ref.read_stimulation(str(p), t2, layer=10)
    np.testing.assert_array_equal(m2, mr2)
    np.testing.assert_array_equal(on2, onr2)


def test_geometry_reader_rejects_bad_input(lq, tmp_path):
    p = tmp_path / "bad.txt"
    p.write_text("1 2 3 0.1 0.2 0.3 5\n1 2 3 0.1 0.2 0.3 5\n")
    with pytest.raises(lq.LqtError):
        lq.geometry.load_geometry(str(p), (10, 10, 10))
    p.write_text("1 2 30 0.1 0.2 0.3 5\n")
    with pytest.raises(lq.LqtError):
        lq.geometry.load_geometry(str(p), (10, 10, 10))
    with pytest.raises(lq.LqtError):
        lq.geometry.load_geometry(str(tmp_path / "missing.txt"), (10, 10, 10))
