"""The learned surrogate's network on the GPU (lqt_mlp_*).

48 -> 128 -> 128 -> 48 MLP with SiLU, BF16 weights, FP32 accumulation.
Inference runs on the tcgen05 tensor cores (TMEM accumulators); training uses
hand-written BF16 mma.sync GEMMs and Adam.  Device buffers are torch tensors
owned by the caller.
"""
from __future__ import annotations

import ctypes as C
import json
import os

import numpy as np

from . import _native as N

IN, HID, OUT = 48, 128, 48
N_STATE, N_PARAM = 38, 6


def _bind():
    L = N.lib()
    P = C.c_void_p
    sig = {
        "lqt_mlp_create": ([C.c_uint64, P, C.POINTER(P)], C.c_int),
        "lqt_mlp_destroy": ([P], None),
        "lqt_mlp_num_params": ([], C.c_int64),
        "lqt_mlp_set_params": ([P, P], C.c_int),
        "lqt_mlp_get_params": ([P, P, P], C.c_int),
        "lqt_mlp_set_norm": ([P, P, P, P, C.c_int32], C.c_int),
        "lqt_mlp_set_bounds": ([P, P], C.c_int),
        "lqt_mlp_set_layout": ([P, C.c_int32], C.c_int),
        "lqt_mlp_infer": ([P, P, P, C.c_int64], C.c_int),
        "lqt_mlp_gradients": ([P, P, P, C.c_int64, C.POINTER(C.c_double)], C.c_int),
        "lqt_mlp_train_step": ([P, P, P, C.c_int64, C.c_float, C.POINTER(C.c_double)], C.c_int),
    }
    for k, (a, r) in sig.items():
        f = getattr(L, k)
        f.argtypes, f.restype = a, r
    return L


class Mlp:
    def __init__(self, seed: int = 0, stream: int | None = None):
        self.L = _bind()
        h = C.c_void_p()
        N.check(self.L.lqt_mlp_create(seed, C.c_void_p(stream or 0), C.byref(h)), "lqt_mlp_create")
        self._h = h
        self.nparam = int(self.L.lqt_mlp_num_params())
        self.nsub = 5       # plain steps per macro step the network was trained for

    def close(self):
        if getattr(self, "_h", None):
            self.L.lqt_mlp_destroy(self._h)
            self._h = None

    __del__ = close

    def params(self):
        p = np.zeros(self.nparam, np.float32)
        N.check(self.L.lqt_mlp_get_params(self._h, p.ctypes.data, None), "lqt_mlp_get_params")
        return p

    def grads(self):
        g = np.zeros(self.nparam, np.float32)
        N.check(self.L.lqt_mlp_get_params(self._h, None, g.ctypes.data), "lqt_mlp_get_params")
        return g

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        N.check(self.L.lqt_mlp_set_params(self._h, p.ctypes.data), "lqt_mlp_set_params")

    def set_norm(self, in_mean, in_scale, out_scale, nvalid=N_STATE):
        a = [np.ascontiguousarray(x, np.float32) for x in (in_mean, in_scale, out_scale)]
        self.norm_in_mean, self.norm_in_scale, self.norm_out = a
        N.check(self.L.lqt_mlp_set_norm(self._h, a[0].ctypes.data, a[1].ctypes.data, a[2].ctypes.data, nvalid),
                "lqt_mlp_set_norm")

    def set_bounds(self, out_bound):
        """Residual bounds (normalised units) for the tissue macro step."""
        b = np.ascontiguousarray(out_bound, np.float32)
        self.out_bound = b
        N.check(self.L.lqt_mlp_set_bounds(self._h, b.ctypes.data), "lqt_mlp_set_bounds")

    def set_layout(self, layout: int):
        N.check(self.L.lqt_mlp_set_layout(self._h, layout), "lqt_mlp_set_layout")

    def infer(self, x_bf16, y_f32):
        """x_bf16: torch bfloat16 [n, 48] cuda; y_f32: torch float32 [n, 48] cuda."""
        N.check(self.L.lqt_mlp_infer(self._h, x_bf16.data_ptr(), y_f32.data_ptr(), x_bf16.shape[0]), "lqt_mlp_infer")

    def gradients(self, x_bf16, t_f32):
        loss = C.c_double()
        N.check(self.L.lqt_mlp_gradients(self._h, x_bf16.data_ptr(), t_f32.data_ptr(), x_bf16.shape[0],
                                         C.byref(loss)), "lqt_mlp_gradients")
        return loss.value

    def train_step(self, x_bf16, t_f32, lr=1e-3):
        loss = C.c_double()
        N.check(self.L.lqt_mlp_train_step(self._h, x_bf16.data_ptr(), t_f32.data_ptr(), x_bf16.shape[0], lr,
                                          C.byref(loss)), "lqt_mlp_train_step")
        return loss.value


class SurRanges(C.Structure):
    _fields_ = [("gks", C.c_double * 2), ("pca", C.c_double * 2), ("iso", C.c_double * 2), ("bcl", C.c_double * 2),
                ("beats_warm", C.c_int32), ("beats_record", C.c_int32), ("dt", C.c_double), ("dvdt_max", C.c_double),
                ("prob", C.c_double), ("jitter", C.c_double), ("nsub", C.c_int32), ("reserved", C.c_int32)]


def _bind_sur():
    L = _bind()
    P = C.c_void_p
    L.lqt_sur_datagen.argtypes = [C.c_int64, C.c_uint64, C.POINTER(SurRanges), P, P, C.c_int64,
                                  C.POINTER(C.c_int64), P]
    L.lqt_sur_datagen.restype = C.c_int
    L.lqt_sur_prepare.argtypes = [P, P, P, P, C.c_int64, P, P]
    L.lqt_sur_prepare.restype = C.c_int
    return L


def generate(ncells=65536, seed=1, cap=20_000_000, *, gks=(0.05, 1.0), pca=(1.0, 2.2), iso=(1.0, 2.0),
             bcl=(400.0, 2000.0), beats_warm=0, beats_record=6, dvdt_max=2.0, prob=0.005, jitter=0.3, dt=0.02,
             nsub=5, stream=None):
    """Training pairs from the plain mixed-form integrator on the GPU.
    Returns torch tensors X [n, 44] (raw features) and D [n, 38] (state after
    nsub plain steps of dt minus the state after one coarse step of nsub * dt)."""
    import torch
    L = _bind_sur()
    X = torch.empty((cap, 44), dtype=torch.float32, device="cuda")
    D = torch.empty((cap, N_STATE), dtype=torch.float32, device="cuda")
    r = SurRanges((C.c_double * 2)(*gks), (C.c_double * 2)(*pca), (C.c_double * 2)(*iso), (C.c_double * 2)(*bcl),
                  beats_warm, beats_record, dt, dvdt_max, prob, jitter, nsub, 0)
    n = C.c_int64()
    N.check(L.lqt_sur_datagen(ncells, seed, C.byref(r), X.data_ptr(), D.data_ptr(), cap, C.byref(n),
                              C.c_void_p(stream or 0)), "lqt_sur_datagen")
    return X[:n.value], D[:n.value]


# network order of the 38 evolving states -> index in the 40-state vector
REF_INDEX = [0] + list(range(1, 9)) + [9 + (j if j < 3 else j + 2) for j in range(29)]


def tissue_pairs(n_target=6_000_000, *, sheets=4, n=160, t_end=900.0, grab_every=2.0, dvdt_max=2.0, seed=7,
                 gks=(0.05, 1.0), pca=(1.0, 2.2), iso=(1.0, 2.0), nsub=5, log=print):
    """Training pairs from tissue: 2D sheets in the layout of the 600 x 600
    S1-S2 workload (n x n at 0.15 mm, endo/M/epi bands, S1 line, S2 quadrant at
    a seeded coupling interval U[300, 360] ms), each with a seeded model, run
    with the plain mixed-form integrator.  Every `grab_every` ms the voxels
    with |dV/dt| <= dvdt_max over the last step are sampled; the targets are
    computed on the GPU from those states exactly as k_sur_datagen computes
    them (nsub plain steps of 0.02 ms minus one coarse step of nsub * 0.02
    ms, no diffusion, no stimulus).  Returns torch tensors X [m, 44], D [m, 38]."""
    import torch

    from . import geometry
    from .cell import TPORdCells
    from .sim import Sim
    rng = np.random.default_rng(seed)
    X, D = [], []
    per_sheet = n_target // sheets
    for k in range(sheets):
        g_ = float(rng.uniform(*gks))
        p_ = float(rng.uniform(*pca))
        i_ = float(rng.uniform(*iso))
        m = N.model("baseline", gks_scale=g_, pca_scale=p_, gks_iso_scale=i_)
        sh = geometry.sheet(n, n, s1_cols=3)
        ci = float(rng.uniform(300.0, 360.0))
        sim = Sim(sh.types, 0.15, precision=N.MIXED, model=m)
        sim.set_protocol(bcl=1000.0, s1_mask=sh.s1_mask, s1_start=0.0, s1_duration=2.0, s1_strength=-52.0,
                         s1_beats=1, s2_time=ci, s2_duration=3.0, s2_strength=-104.0, s2_mask=sh.s2_mask)
        types = sh.types.reshape(-1)[sim.tissue_index()]
        cls = np.where(types == N.EPI, 1, np.where(types == N.MCELL, 2, 0))
        every = int(round(grab_every / 0.02))
        ngrab = int(t_end / grab_every)
        take = min(1.0, per_sheet / (ngrab * sim.n * 0.85))
        sel_states, sel_types, sel_cls = [], [], []
        for _ in range(ngrab):
            sim.step(every - 1)
            v_prev = sim.get_v(as_double=True)
            sim.step(1)
            st = sim.get_state()
            keep = (np.abs((st[:, 0] - v_prev) / 0.02) <= dvdt_max) & (rng.random(sim.n) < take)
            sel_states.append(st[keep])
            sel_types.append(types[keep])
            sel_cls.append(cls[keep])
        sim.close()
        st = np.concatenate(sel_states)
        ty = np.concatenate(sel_types)
        cl = np.concatenate(sel_cls)
        fine = TPORdCells(ty, precision=N.MIXED, model=m, dt=0.02)
        fine.set_state(st)
        fine.update(nsub)
        xf = fine.get_state()
        fine.close()
        coarse = TPORdCells(ty, precision=N.MIXED, model=m, dt=0.02 * nsub)
        coarse.set_state(st)
        coarse.update(1)
        xc = coarse.get_state()
        coarse.close()
        x = np.zeros((len(st), 44), np.float32)
        x[:, :38] = st[:, REF_INDEX]
        x[:, 38:41] = (g_, p_, i_)
        x[np.arange(len(st)), 41 + cl] = 1.0
        X.append(torch.from_numpy(x))
        D.append(torch.from_numpy((xf - xc)[:, REF_INDEX].astype(np.float32)))
        log(f"tissue sheet {k}: model gks {g_:.2f} pca {p_:.2f} iso {i_:.2f}, S2 at {ci:.1f} ms, {len(st)} pairs")
    return torch.cat(X).cuda(), torch.cat(D).cuda()


def fit_bounds(D, out_scale):
    """Largest |normalised target| of each output over the whole set (the
    residual bounds); outputs without a target get 1."""
    import torch
    osc = torch.from_numpy(np.ascontiguousarray(out_scale[:N_STATE], np.float32)).cuda()
    mx = torch.zeros(N_STATE, device="cuda")
    for i in range(0, D.shape[0], 1 << 22):
        mx = torch.maximum(mx, (D[i:i + (1 << 22)].abs() / osc).amax(0))
    b = np.ones(OUT, np.float32)
    b[:N_STATE] = np.maximum(mx.cpu().numpy(), 1e-3)
    return b


def fit_norm(X, D, nsample=500_000, seed=0):
    """Per-feature normalisation from a sample: inputs to zero mean / unit std
    (constant features keep scale 1), targets divided by their std."""
    import torch
    g = torch.Generator(device="cuda").manual_seed(seed)
    idx = torch.randint(0, X.shape[0], (min(nsample, X.shape[0]),), device="cuda", generator=g)
    xs = X[idx].double().cpu().numpy()
    ds = D[idx].double().cpu().numpy()
    in_mean = np.zeros(IN, np.float32)
    in_scale = np.ones(IN, np.float32)
    mu, sd = xs.mean(0), xs.std(0)
    in_mean[:44] = mu
    in_scale[:44] = np.where(sd > 1e-12 * np.maximum(1.0, np.abs(mu)), 1.0 / np.maximum(sd, 1e-30), 1.0)
    out_scale = np.ones(OUT, np.float32)
    out_scale[:N_STATE] = np.maximum(ds.std(0), 1e-12)
    return in_mean, in_scale, out_scale


# Pairs whose V lies in this range (mV) are repolarisation (phase 3) states:
# the upstroke foot and the notch are outside the surrogate's |dV/dt| window.
PHASE3_V = (-80.0, -20.0)


def train(mlp: Mlp, X, D, *, epochs=4, batch=8192, lr=2e-3, lr_min=1e-4, holdout=0.01, seed=0, log_every=500,
          oversample=1, log=print):
    """Adam on shuffled mini-batches with a cosine learning-rate schedule.
    oversample > 1 repeats the training split's phase-3 pairs (V in
    PHASE3_V) that many times per epoch: they are a few percent of the pairs,
    and a small bias of their correction accumulates over the ~100 macro steps
    of repolarisation into the APD.  The held-out tail is never repeated.
    Returns per-state validation RMSE (physical units) and the loss history."""
    import math

    import torch
    L = _bind_sur()
    n = X.shape[0]
    nval = max(batch, int(n * holdout)) // 16 * 16
    ntr = n - nval
    xb = torch.empty((batch, IN), dtype=torch.bfloat16, device="cuda")
    t = torch.empty((batch, OUT), dtype=torch.float32, device="cuda")
    g = torch.Generator(device="cuda").manual_seed(seed)
    tr_idx = torch.arange(ntr, device="cuda")
    if oversample > 1:
        v = X[:ntr, 0]
        sel = torch.nonzero((v > PHASE3_V[0]) & (v < PHASE3_V[1])).squeeze(1)
        tr_idx = torch.cat([tr_idx, sel.repeat(oversample - 1)])
        log(f"phase-3 pairs {int(sel.numel())} of {ntr}, repeated x{oversample}")
    nep = tr_idx.numel() // batch
    steps = epochs * nep
    hist = []
    k = 0
    for ep in range(epochs):
        perm = tr_idx[torch.randperm(tr_idx.numel(), device="cuda", generator=g)]
        for b in range(nep):
            idx = perm[b * batch:(b + 1) * batch]
            N.check(L.lqt_sur_prepare(mlp._h, X.data_ptr(), D.data_ptr(), idx.data_ptr(), batch, xb.data_ptr(),
                                      t.data_ptr()), "lqt_sur_prepare")
            cur = lr_min + 0.5 * (lr - lr_min) * (1 + math.cos(math.pi * k / max(1, steps)))
            if k % log_every == 0 or k == steps - 1:
                loss = mlp.train_step(xb, t, cur)
                hist.append((k, loss))
                log(f"step {k}/{steps} lr {cur:.2e} loss {loss:.3e}")
            else:
                N.check(mlp.L.lqt_mlp_train_step(mlp._h, xb.data_ptr(), t.data_ptr(), batch, cur, None),
                        "lqt_mlp_train_step")
            k += 1
    return validate(mlp, X[ntr:], D[ntr:]), hist


def validate(mlp: Mlp, Xv, Dv, out_scale=None):
    """Per-state RMSE of the predicted correction (physical units) and the
    RMSE of the zero correction (the coarse step alone), on tcgen05 inference."""
    import torch
    L = _bind_sur()
    n = Xv.shape[0]
    xb = torch.empty((n, IN), dtype=torch.bfloat16, device="cuda")
    y = torch.empty((n, OUT), dtype=torch.float32, device="cuda")
    N.check(L.lqt_sur_prepare(mlp._h, Xv.data_ptr(), None, None, n, xb.data_ptr(), None), "lqt_sur_prepare")
    mlp.infer(xb, y)
    os_ = mlp.norm_out if out_scale is None else out_scale
    pred = y[:, :N_STATE].double().cpu().numpy() * os_[:N_STATE]
    true = Dv.double().cpu().numpy()
    rmse = np.sqrt(((pred - true) ** 2).mean(0))
    base = np.sqrt((true ** 2).mean(0))
    return dict(rmse=rmse, zero_rmse=base, n=n)


def validate_tissue(mlp: Mlp, *, n=64, t_end=600.0, dvdt_max=1.0, vstep_max=0.3, ref=None):
    """APD90 error of the surrogate form against the FP64 form on a
    validation tissue that the accuracy tests do not use: an n x n sheet at
    0.15 mm (endo/M/epi bands, S1 on one edge, one beat) with the model GKs
    x0.7, PCa x1.6, GKs-ISO x1.2.  Returns (mean signed error, max |error|,
    the FP64 result for reuse)."""
    from . import geometry
    from .sim import Sim
    sh = geometry.sheet(n, n, s1_cols=3)
    m = N.model("baseline", gks_scale=0.7, pca_scale=1.6, gks_iso_scale=1.2)

    def run(prec, net):
        sim = Sim(sh.types, 0.15, precision=prec, model=m)
        sim.set_protocol(bcl=1000.0, s1_mask=sh.s1_mask, s1_start=0.0, s1_duration=2.0, s1_strength=-52.0,
                         s1_beats=1)
        if net is not None:
            sim.set_surrogate(net, dvdt_max=dvdt_max, vstep_max=vstep_max)
        sim.step(int(round(t_end / 0.02)))
        d = sim.detect()
        sim.close()
        return d["apd90"]
    if ref is None:
        ref = run(N.FP64, None)
    a = run(N.MIXED, mlp)
    ok = (a > 0) & (ref > 0)
    e = (a - ref)[ok]
    if e.size == 0 or ok.sum() < 0.99 * (ref > 0).sum():
        return float("inf"), float("inf"), ref
    return float(e.mean()), float(np.abs(e).max()), ref


DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "tpord_surrogate.npz")


def save(mlp: Mlp, path: str, meta: dict | None = None):
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    np.savez(path, params=mlp.params(), in_mean=mlp.norm_in_mean, in_scale=mlp.norm_in_scale,
             out_scale=mlp.norm_out, out_bound=getattr(mlp, "out_bound", np.full(OUT, np.inf, np.float32)),
             meta=np.array(json.dumps(meta or {})))


def load(path: str | None = None, stream: int | None = None) -> Mlp:
    """A network with the weights and normalisation of a saved file (the
    shipped TPORd surrogate by default)."""
    z = np.load(path or DEFAULT_WEIGHTS)
    m = Mlp(seed=0, stream=stream)
    m.set_params(z["params"])
    m.set_norm(z["in_mean"], z["in_scale"], z["out_scale"])
    if "out_bound" in z.files and np.isfinite(z["out_bound"]).all():
        m.set_bounds(z["out_bound"])
    m.meta = json.loads(str(z["meta"]))
    m.nsub = int(m.meta.get("macro_steps", 5))
    return m


def train_default(out=DEFAULT_WEIGHTS, *, ncells=65536, cap=20_000_000, prob=None, epochs=20, batch=8192,
                  lr=2e-3, seed=1, tissue=0, nsub=10, oversample=4, select=4, jitter=0.3, log=print):
    """Generate the pairs (paced single cells with the sweep's parameter
    ranges, plus `tissue` pairs from 2D S1-S2 sheets), fit the normalisation,
    train `select` networks (seeds seed, seed + 1, ...) on the same pairs,
    keep the one whose APD90 on the validation tissue (validate_tissue) is
    least biased against the FP64 form, save.  Networks with the same
    per-pair loss differ in a small state-dependent bias that shifts every
    cell's APD by up to ~0.5 ms; the squared loss does not see it, the
    tissue does.  Defaults: macro steps of 10 plain steps (0.2 ms), recording
    probability 0.001 * nsub (about cap pairs from 6 beats of 65,536 cells),
    phase-3 pairs repeated 4 times, 20 epochs, best of 4.  The shipped
    network came from this recipe with one candidate and was selected by the
    same validation among the networks trained so far (its file records
    them); a rerun is not bitwise reproducible (the pair generator's slot
    order depends on atomics), so its candidates differ from it."""
    if prob is None:
        prob = 0.001 * nsub
    import time

    import torch
    t0 = time.perf_counter()
    X, D = generate(ncells=ncells, cap=cap - tissue, prob=prob * (cap - tissue) / cap, seed=seed, nsub=nsub,
                    jitter=jitter)
    if tissue > 0:
        Xt, Dt = tissue_pairs(tissue, seed=seed + 6, nsub=nsub, log=log)
        X, D = torch.cat([X, Xt]), torch.cat([D, Dt])
        del Xt, Dt
        # one shuffle, so that the held-out tail mixes both sources
        g = torch.Generator(device="cuda").manual_seed(seed)
        perm = torch.randperm(X.shape[0], device="cuda", generator=g)
        X, D = X[perm], D[perm]
        del perm
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    log(f"pairs {X.shape[0]} ({X.shape[0] - tissue if tissue else X.shape[0]} single-cell) in {t1 - t0:.1f} s")
    im, isc, osc = fit_norm(X, D)
    bounds = fit_bounds(D, osc)
    best, ref, cand = None, None, []
    for i in range(max(1, select)):
        m = Mlp(seed=seed + i)
        m.nsub = nsub
        m.set_norm(im, isc, osc)
        m.set_bounds(bounds)
        val_i, hist_i = train(m, X, D, epochs=epochs, batch=batch, lr=lr, seed=seed + i, oversample=oversample,
                              log=log)
        bias, emax, ref = validate_tissue(m, ref=ref)
        cand.append(dict(seed=seed + i, apd_bias_ms=bias, apd_max_ms=emax))
        log(f"candidate seed {seed + i}: validation APD90 bias {bias:+.3f} ms, max {emax:.3f} ms")
        if best is None or (abs(bias), emax) < (abs(best[1]), best[2]):
            if best is not None:
                best[0].close()
            best = (m, bias, emax, val_i, hist_i, seed + i)
        else:
            m.close()
    m, _, _, val, hist, seed_best = best
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    rel = val["rmse"] / np.maximum(val["zero_rmse"], 1e-30)
    meta = dict(pairs=int(X.shape[0]), tissue_pairs=int(tissue), ncells=ncells, epochs=epochs, batch=batch, lr=lr,
                seed=seed_best, data_seed=seed, dt=0.02, prob=prob, jitter=jitter, oversample_phase3=oversample,
                candidates=cand,
                macro_steps=nsub, gen_s=t1 - t0, train_s=t2 - t1, loss_history=[(int(k), float(l)) for k, l in hist],
                val_rmse=val["rmse"].tolist(), val_zero_rmse=val["zero_rmse"].tolist(), val_n=int(val["n"]),
                state_names=STATE_NAMES)
    save(m, out, meta)
    log(json.dumps({"pairs": meta["pairs"], "gen_s": round(meta["gen_s"], 2), "train_s": round(meta["train_s"], 2),
                    "final_loss": hist[-1][1] if hist else None,
                    "rmse_over_coarse_median": float(np.median(rel)), "rmse_over_coarse_max": float(rel.max()),
                    "v_rmse_mV": float(val["rmse"][0]), "v_coarse_rmse_mV": float(val["zero_rmse"][0])}))
    return m, meta


STATE_NAMES = ["v", "nai", "nass", "ki", "kss", "cai", "cass", "cansr", "cajsr", "m", "h", "j", "mL", "hL", "hLp",
               "a", "iF", "iS", "ap", "iFp", "iSp", "d", "ff", "fs", "fcaf", "fcas", "jca", "nca", "ffp", "fcafp",
               "xrf", "xrs", "xs1", "xs2", "xk1", "Jrelnp", "Jrelp", "CaMKt"]


def main():
    import argparse
    ap = argparse.ArgumentParser(description="Train the TPORd surrogate on the GPU")
    ap.add_argument("what", choices=["train"])
    ap.add_argument("--out", default=DEFAULT_WEIGHTS)
    ap.add_argument("--cells", type=int, default=65536)
    ap.add_argument("--pairs", type=int, default=20_000_000)
    ap.add_argument("--prob", type=float, default=None, help="recording probability (default 0.001 * nsub)")
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--batch", type=int, default=8192)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--tissue", type=int, default=0, help="pairs from 2D S1-S2 sheets mixed in (0 = none)")
    ap.add_argument("--nsub", type=int, default=10, help="plain steps per macro step (divides 50)")
    ap.add_argument("--oversample", type=int, default=4, help="repeats of the phase-3 pairs per epoch")
    ap.add_argument("--select", type=int, default=4, help="networks trained; the least APD-biased is kept")
    a = ap.parse_args()
    train_default(a.out, ncells=a.cells, cap=a.pairs, prob=a.prob, epochs=a.epochs, batch=a.batch, lr=a.lr,
                  seed=a.seed, tissue=a.tissue, nsub=a.nsub, oversample=a.oversample, select=a.select,
                  log=lambda m: print(m, flush=True))


if __name__ == "__main__":
    main()
