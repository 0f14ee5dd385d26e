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


def _grid_ref(orc, dim):
    import ctypes as C
    import os
    path = os.path.join(orc.REF_DIR, f"libgrid_ref_{dim}d.so")
    if not os.path.exists(path):
        pytest.skip("reference build (oracle/_ref) not present on this host")
    L = C.CDLL(path)
    P = C.c_void_p
    L.lqt_ref_map.argtypes = [P]
    L.lqt_ref_dims.argtypes = [P]
    L.lqt_ref_du.argtypes = ([C.c_int, P, P, P, P, P, P, P] if dim == 2 else [C.c_int, P, P, P, P])
    if dim == 2:
        L.lqt_ref_fill_d.argtypes = [C.c_int, C.c_double, C.c_double, P]
    dims = np.zeros(3, np.int32)
    assert L.lqt_ref_dims(dims.ctypes.data) == dim
    return L, tuple(int(d) for d in dims)


def _blob(shape, seed):
    """Random tissue blob with one empty voxel on every grid face."""
    rng = np.random.default_rng(seed)
    g = np.full(shape, 255, np.uint8)
    inner = tuple(slice(1, s - 1) if s > 1 else slice(0, 1) for s in shape)
    sub = tuple(s - 2 if s > 1 else 1 for s in shape)
    g[inner] = np.where(rng.random(sub) < 0.65, rng.integers(2, 5, sub), 255)
    return g


def _ref_g(types, tissue_of, dst, src, pad):
    """The reference's g array after its map loop, from the library's map:
    tissue index + 1 on tissue, -(mirror source + 1) on boundary voxels."""
    want = np.zeros(types.size + pad, np.int32)
    t = tissue_of >= 0
    want[:types.size][t] = tissue_of[t] + 1
    want[dst] = -(tissue_of[src] + 1)
    return want


@pytest.mark.parametrize("dim", [2, 3])
def test_mirror_map_is_the_references_own(orc, dim):
    """The reference's own mirror-map loop (new_11.cu:1535-1689,
    GPU3D.cu:1487-1680, executed on the CPU by oracle/ref_grid_harness.inc)
    gives exactly the library's map on random tissue blobs."""
    from lqt1_gb300 import geometry as G
    L, (X, Y, Z) = _grid_ref(orc, dim)
    shape = (X, Y) if dim == 2 else (X, Y, Z)
    for seed in range(4):
        types = _blob(shape, seed)
        tissue_of, dst, src = G.mirror_map(types)
        pad = Y * Z                        # the extra zero row the 2D loop reads
        g = np.zeros(types.size + pad, np.int32)
        t = types.reshape(-1) != 255
        g[:types.size][t] = np.arange(1, t.sum() + 1)
        L.lqt_ref_map(g.ctypes.data)
        np.testing.assert_array_equal(g, _ref_g(types, tissue_of, dst, src, pad))


@pytest.mark.parametrize("dim", [2, 3])
def test_stencil_matches_the_references_own(orc, dim):
    """The reference's own calc_du (new_11.cu:352-417: 2D anisotropic with the
    dD/dx terms of its D array, new_11.cu:1496-1499; GPU3D.cu:370-385: 3D
    isotropic), executed on the CPU, against the oracle's stencil on the same
    V, fibres and mirror map: equal to the last bits of the sum order."""
    L, (X, Y, Z) = _grid_ref(orc, dim)
    shape = (X, Y) if dim == 2 else (X, Y, Z)
    rng = np.random.default_rng(11 + dim)
    types = _blob(shape, 20 + dim)
    t = types.reshape(-1) != 255
    n = int(t.sum())
    v = rng.uniform(-90.0, 30.0, n)
    pad = Y * Z
    g = np.zeros(types.size + pad, np.int32)
    g[:types.size][t] = np.arange(1, n + 1)
    L.lqt_ref_map(g.ctypes.data)
    rev_g = np.zeros(n + 1, np.int32)
    rev_g[1:] = np.flatnonzero(t)
    du_ref = np.zeros(n)
    m = orc.model("default")
    if dim == 2:
        ang = rng.uniform(-np.pi, np.pi, types.size).astype(np.float32)
        fib = np.stack([np.cos(ang), np.sin(ang), np.zeros_like(ang)], 1).astype(np.float32)
        xx = fib[t, 0].astype(np.float64)
        yy = fib[t, 1].astype(np.float64)
        d = np.zeros(5 * n)
        for k in range(n):
            L.lqt_ref_fill_d(k, xx[k], yy[k], d.ctypes.data)
        L.lqt_ref_du(n, d.ctypes.data, v.ctypes.data, xx.ctypes.data, yy.ctypes.data, du_ref.ctypes.data,
                     g.ctypes.data, rev_g.ctypes.data)
        og = orc.Grid(types, 0.2, fibre=fib.reshape(shape + (3,)), d_f=0.154, d_t=0.0385)
    else:
        L.lqt_ref_du(n, v.ctypes.data, du_ref.ctypes.data, g.ctypes.data, rev_g.ctypes.data)
        og = orc.Grid(types, 0.2, fibre=None, d_f=0.154, d_t=0.154)
    state = orc.initial_state(-87.5, n)
    state[:, 0] = v
    du = og.step(state, m, 0.02)
    scale = np.abs(du_ref).max()
    assert scale > 1.0
    np.testing.assert_allclose(du, du_ref, rtol=0, atol=1e-12 * scale)
