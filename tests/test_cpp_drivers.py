"""The reference's host programs rewritten in C++ against include/lqt.h
(tests/cpp/drivers.cpp): they compile with g++ alone, and on a GPU they give
the same results as the Python path through the same library."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def drivers(tmp_path_factory):
    import lqt1_gb300 as lq
    lq.lib()                               # builds the library if needed
    libdir = os.path.join(ROOT, "lqt1_gb300", "_lib")
    exe = str(tmp_path_factory.mktemp("cpp") / "drivers")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "drivers.cpp"), "-L", libdir, "-llqt",
                        "-Wl,-rpath," + libdir, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_driver_builds_and_reports_usage(drivers):
    r = subprocess.run([drivers], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


@pytest.mark.gpu
def test_oned_driver_matches_python(drivers, tmp_path):
    import lqt1_gb300 as lq
    out = tmp_path / "VentOneDResults.dat"
    r = subprocess.run([drivers, "oned", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    res = lq.OneDStrand(model="default", precision=lq.FP64).run()
    ref = tmp_path / "ref.dat"
    lq.protocols.write_oned_dat(str(ref), res["rec_t"], res["rec"])
    assert out.read_text() == ref.read_text()
    cv = float(r.stdout.split()[1])
    assert abs(cv - res["cv"]) < 1e-6


@pytest.mark.gpu
def test_tissue_driver_reads_reference_files(drivers, tmp_path):
    """Geometry and stimulation profile written in the reference's text
    formats, read and run by the C++ program; the Python path on the same
    files gives bit-identical V."""
    import lqt1_gb300 as lq
    v = lq.geometry.ventricle(nx=44, ny=44, nz=50, dx=0.2, a_out=4.0, c_out=8.0, wall=2.0, z_base=9.0,
                              island_radius=1.5, stim_radius=1.2)
    code_of = {lq.ENDO: 11, lq.EPI: 17, lq.MCELL: 15}
    pts = np.argwhere(v.types != 255)
    with open(tmp_path / "geom.txt", "w") as f:
        f.write("\n".join("%d %d %d %.6f %.6f %.6f %d" % (x, y, z, *v.fibre[x, y, z], code_of[int(v.types[x, y, z])])
                          for x, y, z in pts))
    sp = np.argwhere(v.s1_mask > 0)
    with open(tmp_path / "stim.cnd", "w") as f:
        f.write("\n".join("%d %d %d 0 0 0 %.3f s" % (x, y, z, 0.25 * (z % 4)) for x, y, z in sp))
    steps = 1500
    r = subprocess.run([drivers, "tissue", str(tmp_path / "geom.txt"), str(tmp_path / "stim.cnd"),
                        *map(str, v.types.shape), str(steps), str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    v_cpp = np.fromfile(tmp_path / "v_final.bin")
    g = lq.geometry.load_geometry(str(tmp_path / "geom.txt"), v.types.shape, case_edits=False)
    np.testing.assert_array_equal(g.types, v.types)
    s1, onset = lq.geometry.load_stimulation(str(tmp_path / "stim.cnd"), g.types)
    sim = lq.Sim(g.types, 0.2, fibre=g.fibre, precision=lq.MIXED, model="lqt1")
    sim.set_protocol(bcl=500.0, s1_mask=s1, s1_start=0.0, s1_duration=2.0, s1_strength=-52.0, s1_onset=onset)
    for k in range(0, steps, 500):
        sim.step(min(500, steps - k))
    v_py = sim.get_v(as_double=True)
    np.testing.assert_array_equal(v_cpp, v_py)
    assert (v_py > -30).any()                         # the stimulated wave is on its way
    frames = sorted(p for p in os.listdir(tmp_path) if p.startswith("ap_") and p.endswith(".vtk"))
    assert frames == ["ap_%d.vtk" % (k // 50) for k in range(0, steps, 500)]


@pytest.mark.gpu
def test_single_cell_driver_through_cell_interface(drivers, orc, tmp_path):
    """SingleCell.cc's loop in C++ through lqt_cells_* (setIstim, update,
    getV, getICaL, getIKs, getAbsDvdt, outputAllStates, readinAllStates):
    one beat of an M cell against the FP64 oracle's update and getters."""
    out, states = tmp_path / "single.dat", tmp_path / "states.dat"
    steps = 20000
    r = subprocess.run([drivers, "single", str(out), str(states), str(steps)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = np.loadtxt(out)
    assert rows.shape == (steps, 4)
    # oracle: the same stimulus protocol, one update at a time
    s = orc.initial_state(-87.5)
    m = orc.model("default")
    want = np.zeros((steps, 3))
    dvdt_max = 0.0
    for k in range(steps):
        tb = rows[k, 0] - np.floor(rows[k, 0] / 1000.0) * 1000.0
        ist = np.array([-53.0 if 50.0 <= tb < 51.0 else 0.0])
        cur = orc.cells_currents(s, [orc.MCELL], m, ist=ist)[0]
        want[k] = s[0, 0], cur[1], cur[3]
        dvdt_max = max(dvdt_max, cur[5])
    assert np.abs(rows[:, 1] - want[:, 0]).max() < 1e-3          # V, mV (printed to 1e-10)
    scale = np.abs(want[:, 1:]).max(axis=0)
    assert (np.abs(rows[:, 2:] - want[:, 1:]).max(axis=0) < 1e-4 * scale).all()
    got_max = float(r.stdout.split()[1])
    assert abs(got_max - dvdt_max) < 1e-6 * dvdt_max
    assert len(open(states).read().split()) == 40
