"""Whole-beat tissue parity against the CPU oracle itself.

A small anisotropic sheet and a small ventricle-shaped shell are run for one
beat (S1 at t = 0, 450 ms: upstroke, plateau, repolarisation and rest) by the
FP64 oracle (oracle/lqt_oracle.c through tests/grid_ref.py) and on the GPU in
the FP64 form, the mixed form and the FP32 + surrogate form.  Each GPU form
is held to the bars the reference's own FP64 CPU path sets for the build:
activation within 0.1 ms, APD90 within 1 ms at every voxel, V within 0.5 mV
outside the upstroke.  The FP64 form is held far tighter.
"""
import os

import numpy as np
import pytest

from grid_ref import run_oracle_grid

pytestmark = pytest.mark.gpu

NSTEPS = 22500           # 450 ms of 0.02 ms steps
REC = 100                # V recorded every 2 ms


@pytest.fixture(scope="module")
def lq():
    import lqt1_gb300 as lq
    lq.lib()
    return lq


@pytest.fixture(scope="module")
def net(lq):
    from lqt1_gb300 import surrogate as S
    if not os.path.exists(S.DEFAULT_WEIGHTS):
        pytest.fail("trained surrogate weights missing: " + S.DEFAULT_WEIGHTS)
    return S.load()


def tissue(lq, case):
    if case == "sheet":
        sh = lq.geometry.sheet(24, 24, s1_cols=2)
        nx, ny = sh.types.shape
        ang = np.linspace(-0.8, 0.8, ny)[None, :].repeat(nx, 0)
        fib = np.zeros((nx, ny, 3), np.float32)
        fib[..., 0] = np.cos(ang)
        fib[..., 1] = np.sin(ang)
        return sh.types, sh.s1_mask, fib, 0.15
    v = lq.geometry.ventricle(nx=22, ny=22, nz=26, dx=0.2, a_out=1.9, c_out=4.2, wall=1.0, z_base=4.6,
                              island_radius=0.6, stim_radius=0.6)
    return v.types, v.s1_mask, v.fibre, 0.2


def model_pair(lq, orc):
    # the 3D workload's model: IKs x0.5, ICaL x2, IKs-ISO x1.5
    kw = dict(gks_scale=0.5, pca_scale=2.0, gks_iso_scale=1.5)
    return lq.model("baseline", **kw), orc.model("baseline", **kw)


@pytest.fixture(scope="module", params=["sheet", "shell"])
def case(request, lq, orc):
    types, s1, fib, dx = tissue(lq, request.param)
    _, om = model_pair(lq, orc)
    og = orc.Grid(types, dx, fibre=fib)
    ref = run_oracle_grid(orc, og, om, NSTEPS, s1_mask=s1, s1_dur=2.0, s1_beats=1, record_every=REC, detect=True)
    return request.param, types, s1, fib, dx, ref


def run_gpu(lq, types, s1, fib, dx, m, precision, net=None):
    sim = lq.Sim(types, dx, fibre=fib, precision=precision, model=m)
    sim.set_protocol(bcl=1000.0, s1_mask=s1, s1_start=0.0, s1_duration=2.0, s1_strength=-52.0, s1_beats=1)
    if net is not None:
        sim.set_surrogate(net)
    recs = []
    for _ in range(NSTEPS // REC):
        sim.step(REC)
        recs.append(sim.get_v(as_double=True))
    out = dict(rec=np.array(recs), det=sim.detect(), bad=sim.check(),
               stats=sim.surrogate_stats() if net is not None else None)
    sim.close()
    return out


def errors(got, ref):
    t_act = ref["t_act_last"]
    assert (t_act >= 0).all() and (ref["apd90"] > 0).all()     # every voxel activates and repolarises
    d = got["det"]
    assert (d["t_act"] >= 0).all() and (d["apd90"] > 0).all()
    ts = REC * 0.02 * np.arange(1, NSTEPS // REC + 1)
    # outside the upstroke: record times not within [t_act - 1, t_act + 5] ms
    calm = ~((ts[:, None] >= t_act[None, :] - 1.0) & (ts[:, None] <= t_act[None, :] + 5.0))
    return dict(act=float(np.abs(d["t_act"] - t_act).max()), apd=float(np.abs(d["apd90"] - ref["apd90"]).max()),
                v=float(np.abs(got["rec"] - ref["rec"])[calm].max()))


def test_fp64_form_whole_beat(lq, orc, case):
    name, types, s1, fib, dx, ref = case
    m, _ = model_pair(lq, orc)
    got = run_gpu(lq, types, s1, fib, dx, m, lq.FP64)
    assert got["bad"] == 0
    e = errors(got, ref)
    # CUDA vs glibc last-bit differences of exp/log: one step of detector time
    # at most, microvolts in V
    assert e["act"] <= 0.02 + 1e-4 and e["apd"] <= 0.04 + 1e-4 and e["v"] < 0.01, (name, e)


def test_mixed_form_whole_beat(lq, orc, case):
    name, types, s1, fib, dx, ref = case
    m, _ = model_pair(lq, orc)
    got = run_gpu(lq, types, s1, fib, dx, m, lq.MIXED)
    assert got["bad"] == 0
    e = errors(got, ref)
    assert e["act"] <= 0.1 + 1e-4 and e["apd"] <= 1.0 and e["v"] < 0.5, (name, e)


def test_surrogate_form_whole_beat(lq, orc, net, case):
    name, types, s1, fib, dx, ref = case
    m, _ = model_pair(lq, orc)
    got = run_gpu(lq, types, s1, fib, dx, m, lq.MIXED, net)
    assert got["bad"] == 0 and got["stats"]["wait_timeouts"] == 0
    # the network carried most of the beat
    assert got["stats"]["accepted"] > 0.5 * got["stats"]["macro_steps"] * len(ref["apd90"])
    e = errors(got, ref)
    assert e["act"] <= 0.1 + 1e-4 and e["apd"] <= 1.0 and e["v"] < 0.5, (name, e)
