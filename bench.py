"""Benchmark of the monodomain TPORd step on the 3D ventricle-shaped workload.

One "step" advances every tissue voxel of the workload by dt = 0.02 ms:
stimulus + anisotropic diffusion + TPORd ionic update + V update +
activation / APD90 detectors, with the pseudo-ECG of 6 electrodes sampled
every 50 steps.  The metric is cell-steps/s (voxels x steps / s).

Default: 3D truncated prolate-ellipsoid shell in a 320x320x420 grid at
0.2 mm (about 7.1M tissue voxels), fibres +60 -> -60 degrees, IKs x0.5,
beta-adrenergic ICaL x2 / IKs x1.5, apical stimulus at BCL 800 ms, timed over
one whole beat (40000 steps).  The headline form is FP32 + learned surrogate
(0.2 ms macro steps of a coarse TPORd step plus a BF16 tensor-core network's
correction where |dV/dt| <= 1.5 mV/ms; plain steps elsewhere).  Beside it: the
plain mixed form over the same steps, the plain FP64 form, the APD90 /
activation error of both FP32 forms against FP64 on a 100k-voxel shell over a
beat, the batched sweep, and the CPU oracle on a slab of the workload.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload ventricle3d|ventricle3d_small|sheet2d]

Under torchrun each rank runs an independent replica (the path has no data
exchange between instances); value = voxel-steps of all ranks / max time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "monodomain cell-steps/s: plain FP64 vs FP32/surrogate form at ≤1 ms APD90 err"
UNIT = "cell-steps/s"
# algorithmic bytes per voxel-step of the fused step kernel (k_grid_step):
# state read+write (8 concentrations as Kahan FP32 pairs or FP64, 29 evolving
# gates/fluxes), own V read + write, tissue->grid index, control byte,
# diffusion tensor (6) and its divergence (3), AP-detector record (16 B read)
BYTES_MIXED = 8 * 8 * 2 + 29 * 4 * 2 + 4 + 4 + 4 + 1 + 9 * 4 + 16
BYTES_FP64 = 8 * 8 * 2 + 29 * 8 * 2 + 8 + 8 + 4 + 1 + 9 * 8 + 16
# surrogate macro-step kernel (k_sur_grid), per voxel per launch: V now and
# one step back, grid index, control byte, detector record, the state read
# once and written once (8 Kahan pairs + 29 gates), the macro step's rate
BYTES_SUR_MACRO = 4 + 4 + 4 + 1 + 16 + (8 * 8 + 29 * 4) * 2 + 4
# and the network's multiply-adds (48 -> 128 -> 128 -> 48) per voxel
FLOP_SUR_MACRO = 2 * (48 * 128 + 128 * 128 + 128 * 48)
# surrogate acceptance thresholds passed to every set_surrogate call (set
# from the command line in main)
SUR_CFG = {}


def workload_model():
    import lqt1_gb300 as lq
    # IKs x0.5 (LQT1), beta-adrenergic ICaL x2 / IKs x1.5, no gate shifts
    return lq.model("baseline", gks_scale=0.5, pca_scale=2.0, gks_iso_scale=1.5)


def build_workload(name):
    import lqt1_gb300 as lq
    if name in ("ventricle3d", "ventricle3d_small"):
        v = lq.geometry.ventricle() if name == "ventricle3d" else lq.geometry.ventricle(
            nx=170, ny=170, nz=220, a_out=14.0, c_out=36.0, wall=6.0, z_base=40.0, island_radius=4.0,
            stim_radius=2.0)
        # six electrodes around the mid-height, 20 mm outside the epicardium
        cx, cy = v.spec.cx, v.spec.cy
        zm = v.spec.z_base - 0.5 * v.spec.c_out
        r = v.spec.a_out + 20.0
        el = [(cx + r * math.cos(a), cy + r * math.sin(a), zm) for a in np.linspace(0, 2 * math.pi, 7)[:-1]]
        nt = int((v.types != 255).sum())
        return dict(types=v.types, fibre=v.fibre, s1=v.s1_mask, dx=0.2, bcl=800.0, electrodes=el,
                    desc="3d-ventricle %dx%dx%d @0.2mm, %d tissue voxels" % (v.types.shape + (nt,)))
    sh = lq.geometry.sheet(600, 600)
    return dict(types=sh.types, fibre=None, s1=sh.s1_mask, s2=sh.s2_mask, dx=0.15, bcl=1000.0,
                electrodes=[(45.0, 45.0, 10.0)], desc="2d-sheet 600x600 @0.15mm")


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms from before
    the headline until the last GPU leg ends; the samples that fall inside the
    headline's timed windows are summarised on their own."""

    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int, path: str | None = None):
        import tempfile
        self.device = device
        self.proc = None
        self.windows = []          # (t0, t1) epoch seconds of the timed windows
        self.path = path or os.path.join(tempfile.gettempdir(), f"lqt_bench_clocks_rank{device}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, ValueError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    @staticmethod
    def _rows(text):
        import datetime
        out = []
        for r in text.strip().splitlines():
            f = [x.strip() for x in r.split(",")]
            if len(f) < 10:
                continue
            try:
                ts = datetime.datetime.strptime(f[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                sm, mx = float(f[2]), float(f[3])
            except ValueError:
                continue
            out.append((ts, sm, mx, f[6:10]))
        return out

    def summary(self):
        try:
            rows = self._rows(open(self.path).read())
        except OSError:
            return None
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

        def summ(rs):
            if not rs:
                return None
            return {"sm_mhz": statistics.median(r[1] for r in rs), "sm_max_mhz": max(r[2] for r in rs),
                    "reasons": sorted({names[i] for r in rs for i in range(4) if r[3][i] == "Active"}),
                    "samples": len(rs)}
        inside = [r for r in rows if any(a - 0.1 <= r[0] <= b + 0.1 for a, b in self.windows)]
        out = summ(rows)
        out["span"] = "every GPU leg of this run, 200 ms samples"
        out["headline_windows"] = summ(inside)
        return out


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return {}


def traffic_summary(name):
    """Per-launch DRAM bytes of a kernel from its committed ncu summary."""
    p = os.path.join(ROOT, "profiles", name)
    try:
        d = json.load(open(p))
        return d.get("traffic_bytes_per_launch_full_workload")
    except (OSError, ValueError):
        return None


# ---------------------------------------------------------------------------
def cpu_sample(w, max_voxels=200_000):
    """A bounded sample of the workload for the CPU oracle: a slab of the grid
    (full y, z; a range of x planes) with ~max_voxels tissue voxels, its faces
    emptied so the oracle grid is valid."""
    t = w["types"]
    per_x = (t != 255).reshape(t.shape[0], -1).sum(1)
    x0 = int(np.argmax(per_x > 0))
    x1 = x0
    tot = 0
    while x1 < t.shape[0] and tot < max_voxels:
        tot += per_x[x1]
        x1 += 1
    sl = slice(max(0, x0 - 1), min(t.shape[0], x1 + 1))
    sub = t[sl].copy()
    sub[0] = 255
    sub[-1] = 255
    fib = None if w["fibre"] is None else np.ascontiguousarray(w["fibre"][sl])
    return sub, fib


def run_cpu(w, steps, warmup, seconds=None, threads=None, max_voxels=200_000):
    """The FP64 oracle (restatement of TPORd.cc + the 3D diffusion) on a slab
    of the workload, OpenMP over voxels on `threads` host threads (default:
    all cores)."""
    from oracle import orc
    orc.build()
    sub, fib = cpu_sample(w, max_voxels)
    og = orc.Grid(sub, w["dx"], fibre=fib)
    m = orc.model(dict(dss_shift=0, fss_shift=0, pca_scale=2.0, gks_scale=0.5, gks_iso_scale=1.5, suprep_dose=0))
    st = orc.initial_state(-87.5, og.n)
    cores = threads or os.cpu_count() or 1
    for _ in range(warmup):
        og.step(st, m, 0.02, None, cores)
    t0 = time.perf_counter()
    done = 0
    while done < steps and (seconds is None or time.perf_counter() - t0 < seconds or done < 3):
        og.step(st, m, 0.02, None, cores)
        done += 1
    el = time.perf_counter() - t0
    return dict(value=og.n * done / el, cores=cores, n=og.n, steps=done, seconds=el)


def cpu_model_name():
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


# phase windows of the beat (ms after the S1 at t = 0) timed when --steps is
# shorter than a beat: the wavefront still sweeping the ventricle, the
# plateau, repolarisation, rest
PHASES = (("upstroke", 20.0), ("plateau", 150.0), ("repolarisation", 330.0), ("rest", 600.0))
SUR_AT_SPEC = dict(dvdt_max=1.0, vstep_max=0.3)      # config 5 as stated: 1 mV/ms gate
AT_SPEC_WEIGHTS = os.path.join(ROOT, "lqt1_gb300", "data", "tpord_surrogate_nsub5.npz")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40000,
                    help="timed steps: one 800 ms beat by default; fewer are timed at each of four phases")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ventricle3d", choices=["ventricle3d", "ventricle3d_small", "sheet2d"])
    ap.add_argument("--prerun", type=int, default=0, help="untimed steps before the timed region (setup)")
    ap.add_argument("--weights", default=None, help="surrogate network file (default: the shipped network)")
    ap.add_argument("--clocks-csv", default=None, help="where to keep the raw nvidia-smi samples (default: temp dir)")
    ap.add_argument("--substep-variant", type=int, default=-1,
                    help="force the surrogate substep kernel (5/6/8 direct, 105/106/108 staged rows, "
                         "203/204 staged rows and V halo, 304/305/306 rows from a producer warp; -1 = autotune)")
    ap.add_argument("--sur-dvdt-max", type=float, default=1.5, help="surrogate eligibility: |dV/dt| bound, mV/ms")
    ap.add_argument("--sur-vstep-max", type=float, default=0.4, help="surrogate residual check: ionic dV per macro step")
    ap.add_argument("--sur-foot-dvdt", type=float, default=0.1,
                    help="surrogate wave-foot gate: no macro step where V < -40 mV rises faster than this (0 = off)")
    ap.add_argument("--fp64-steps", type=int, default=10)
    ap.add_argument("--mixed-steps", type=int, default=-1, help="steps of the plain mixed leg (-1 = --steps)")
    ap.add_argument("--no-accuracy", dest="accuracy", action="store_false")
    ap.add_argument("--accuracy-ms", type=float, default=460.0,
                    help="simulated ms of the accuracy leg (the 1.35M-voxel shell repolarises by 402 ms)")
    ap.add_argument("--no-configs", dest="configs", action="store_false",
                    help="skip the config 1 (OneD strand) and config 2 (2D sheet) legs")
    ap.add_argument("--no-at-spec", dest="at_spec", action="store_false",
                    help="skip the config-5-as-stated leg (0.1 ms network, 1 mV/ms gate)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sweep-beats", type=int, default=20,
                    help="beats of the 4096-instance batched sweep leg (0 = skip; 20 = the stated sweep)")
    ap.add_argument("--only", default=None, choices=["fp64", "mixed", "surrogate"],
                    help="profiling entry: run --prerun then --steps steps of one form only and print its timing")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return
        w = build_workload(args.workload)
        r = run_cpu(w, args.steps, args.warmup, seconds=60.0)
        cb = {"value": r["value"], "unit": UNIT, "cores": r["cores"], "kind": "port",
              "sample": f"{r['n']} tissue voxels of the workload (x-slab), {r['steps']} steps, oracle FP64 "
                        f"restatement of TPORd.cc + 3D diffusion, OpenMP, {cpu_model_name()}"}
        line = {"metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": args.gpus, "steps": r["steps"],
                "warmup": args.warmup, "ms_per_step": 1e3 * r["seconds"] / r["steps"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": w["desc"] + " (CPU sample)", "l2": "n/a (CPU)"}, "impl": "reference",
                "cpu_baseline": cb, "e2e": {"value": r["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                                            "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import torch
    import lqt1_gb300 as lq
    from lqt1_gb300 import replicas
    from lqt1_gb300 import surrogate as S

    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.cuda.current_device()
    w = build_workload(args.workload)
    stream = torch.cuda.Stream()
    net = S.load(args.weights, stream=stream.cuda_stream)
    SUR_CFG.update(dvdt_max=args.sur_dvdt_max, vstep_max=args.sur_vstep_max, foot_dvdt=args.sur_foot_dvdt,
                   foot_v=-40.0)
    beat = int(round(w["bcl"] / 0.02))
    phase_mode = args.steps < beat
    phases = PHASES if phase_mode else (("beat", None),)

    def make_sim(precision, surrogate, mlp=None, cfg=None):
        sim = lq.Sim(w["types"], w["dx"], fibre=w["fibre"], precision=precision, model=workload_model(),
                     detect=True, vmin_ok=-200.0, vmax_ok=200.0, stream=stream.cuda_stream)
        sim.set_protocol(bcl=w["bcl"], s1_mask=w["s1"], s1_start=0.0, s1_duration=2.0, s1_strength=-52.0,
                         s1_beats=3, s2_time=-1.0)
        sim.set_electrodes(np.array(w["electrodes"]), every=50)
        if surrogate:
            sim.set_surrogate(mlp or net, **(cfg or SUR_CFG))
        return sim

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def timed(sim, steps, clk=None):
        """CUDA-event time of `steps` steps on the simulation's stream, max over ranks."""
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        torch.cuda.synchronize()
        t_wall = time.time()
        e0.record(stream)
        sim.step(steps)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        if clk is not None:
            clk.windows.append((t_wall, time.time()))
        _, ms, _ = replicas.aggregate_throughput(float(sim.n) * steps, e0.elapsed_time(e1))
        return ms

    def advance_to(sim, t_ms):
        """Untimed steps (graph replays) up to the step of time t_ms."""
        k = int(round(t_ms / 0.02)) - int(round(sim.time / 0.02))
        if k > 0:
            sim.step(k)

    def run_phases(sim, k, clk=None, surrogate=False):
        """Time k steps in each window; returns (total ms, per-window dict)."""
        tot, out = 0.0, {}
        for name, t0 in phases:
            if t0 is not None:
                advance_to(sim, t0)
            st0 = sim.surrogate_stats() if surrogate else None
            ms_i = timed(sim, k, clk)
            tot += ms_i
            out[name] = {"t_ms": round(sim.time - k * 0.02, 2), "ms": ms_i,
                         "value": world * sim.n * k / (ms_i / 1e3)}
            if surrogate:
                st1 = sim.surrogate_stats()
                mac = st1["macro_steps"] - st0["macro_steps"]
                out[name]["macro_steps"] = mac
                out[name]["accepted_frac"] = (st1["accepted"] - st0["accepted"]) / max(1, mac * sim.n)
        return tot, out

    if args.only:
        prec = lq.FP64 if args.only == "fp64" else lq.MIXED
        so = make_sim(prec, args.only == "surrogate")
        if args.only == "surrogate" and args.substep_variant >= 0:
            so.substep_variant(args.substep_variant)
        so.step(args.prerun)
        ms_o = timed(so, args.steps)
        print(json.dumps({"only": args.only, "workload": w["desc"], "steps": args.steps, "ms": ms_o,
                          "cell_steps_per_s": so.n * args.steps / (ms_o / 1e3), "blowup_voxel_steps": so.check()}))
        so.close()
        return

    clk = ClockSampler(dev, args.clocks_csv)
    clk.__enter__()
    try:
        # ---- headline: FP32 + surrogate form -------------------------------
        sim = make_sim(lq.MIXED, True)
        n = sim.n
        sim.step(args.prerun)
        if args.substep_variant >= 0:
            sim.substep_variant(args.substep_variant)
        variant, tune_ms = sim.tune(-1)          # occupancy variant of the plain step kernel
        sub_variant, sub_ms = sim.substep_variant(-1, timings=True)   # and of the V-only substep
        sim.step(args.warmup)
        sim.surrogate_stats(reset=True)
        ms, per_phase = run_phases(sim, args.steps, clk, surrogate=True)
        ktot = args.steps * len(phases)
        value = world * n * ktot / (ms / 1e3)
        nbad = sim.check()
        sst = sim.surrogate_stats()
        ms_sub, ms_ghost_s, ms_sur = sim.profile(10)
        sim.close()
        peaks = measured_peaks()
        peak = peaks.get("hbm_gbs")
        peak_kind = "measured" if peak else "fallback"
        peak = peak or 6800.0
        tpeak = peaks.get("bf16_tflops_sustained") or peaks.get("bf16_tflops") or 1700.0
        # dominant kernel of the surrogate form: the macro-step kernel (one launch
        # per macro step), algorithmic bytes and tensor FLOPs per voxel per launch
        ach_sur = BYTES_SUR_MACRO * n / (ms_sur / 1e3) / 1e9
        roof = {"bound": "hbm", "achieved": ach_sur, "peak": peak, "unit": "GB/s", "frac": ach_sur / peak,
                "traffic": traffic_summary("k_sur_grid_ventricle3d.json"), "kernel": "k_sur_grid",
                "kernel_ms": ms_sur, "bytes_per_voxel_launch": BYTES_SUR_MACRO, "peak_source": peak_kind,
                "tensor": {"achieved_tflops": FLOP_SUR_MACRO * n / (ms_sur / 1e3) / 1e12, "peak_tflops": tpeak,
                           "frac": FLOP_SUR_MACRO * n / (ms_sur / 1e3) / 1e12 / tpeak,
                           "flop_per_voxel_launch": FLOP_SUR_MACRO},
                "substep": {"kernels": "k_sur_substep + k_grid_step over the plain-voxel list", "ms": ms_sub,
                            "ghost_ms": ms_ghost_s}}
        surrogate = {"macro_steps": sst["macro_steps"], "voxel_offers": sst["offered"], "accepted": sst["accepted"],
                     "accepted_frac_of_voxel_macro_steps": sst["accepted"] / max(1, sst["macro_steps"] * n),
                     "span": "t = 0 to the end of the last timed window" if phase_mode else "the timed beat",
                     "wait_timeouts": sst["wait_timeouts"], "network": {k: net.meta.get(k) for k in
                                                                       ("pairs", "unique_pairs", "epochs",
                                                                        "oversample_phase3", "gen_and_train_s")}}

        e2e = e2e_leg(lq, torch, make_sim, stream, phases, args.steps, world, variant, sub_variant, advance_to)

        # ---- plain mixed form over the same windows --------------------------
        mixed = None
        if args.mixed_steps != 0:
            ksteps = args.steps if args.mixed_steps < 0 else args.mixed_steps
            sm = make_sim(lq.MIXED, False)
            sm.step(args.prerun)
            variant_m, tune_m = sm.tune(-1)
            sm.step(args.warmup)
            ms_m, per_m = run_phases(sm, ksteps)
            ms_step, ms_ghost, _ = sm.profile(20)
            ach = BYTES_MIXED * n / (ms_step / 1e3) / 1e9
            v_m = world * n * ksteps * len(phases) / (ms_m / 1e3)
            mixed = {"value": v_m, "unit": UNIT, "steps": ksteps, "windows": per_m, "surrogate_over_mixed": value / v_m,
                     "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                                  "traffic": traffic_summary("k_grid_step_ventricle3d.json"),
                                  "kernel": "k_grid_step<float,3>", "kernel_ms": ms_step,
                                  "bytes_per_cell_step": BYTES_MIXED, "peak_source": peak_kind},
                     "step_kernel_variant": {"min_ctas_per_sm": variant_m,
                                             "tuned_ms": [round(float(x), 4) for x in tune_m[:3]]},
                     "blowup_voxel_steps": sm.check()}
            # the same state for the FP64 leg: the plateau or the end of the beat
            st_fp64 = sm.get_state()
            sm.close()

        # ---- plain FP64 form on the same state ----------------------------------
        fp64 = None
        if args.fp64_steps > 0:
            s64 = make_sim(lq.FP64, False)
            if mixed is not None:
                s64.set_state(st_fp64)
                del st_fp64
            s64.step(2)
            ms64t = timed(s64, args.fp64_steps)
            v64 = n * args.fp64_steps / (ms64t / 1e3)
            ms64, _, _ = s64.profile(2)
            fp64 = {"value": v64 * world, "unit": UNIT, "steps": args.fp64_steps, "kernel_ms": ms64,
                    "achieved_gbs": BYTES_FP64 * n / (ms64 / 1e3) / 1e9,
                    "surrogate_over_fp64": value / (v64 * world),
                    "profile": "profiles/k_grid_step_fp64_ventricle3d_small.md"}
            s64.close()

        # ---- config 5 as stated: 0.1 ms network, 1 mV/ms gate, 0.3 mV -------------
        net5 = None
        at_spec = None
        if args.at_spec and os.path.exists(AT_SPEC_WEIGHTS):
            net5 = S.load(AT_SPEC_WEIGHTS, stream=stream.cuda_stream)
            cfg5 = dict(SUR_AT_SPEC, nsub=net5.nsub)
            s5 = make_sim(lq.MIXED, True, net5, cfg5)
            s5.tune(variant)
            s5.substep_variant(sub_variant)
            s5.step(args.warmup)
            s5.surrogate_stats(reset=True)
            ms5, per5 = run_phases(s5, args.steps, surrogate=True)
            st5 = s5.surrogate_stats()
            v5 = world * n * args.steps * len(phases) / (ms5 / 1e3)
            at_spec = {"value": v5, "unit": UNIT, "windows": per5,
                       "form": "0.1 ms macro steps (network trained for nsub = 5), |dV/dt| <= 1 mV/ms, "
                               "ionic dV <= 0.3 mV per macro step, wave-foot gate as the headline's",
                       "accepted_frac_of_voxel_macro_steps": st5["accepted"] / max(1, st5["macro_steps"] * n),
                       "over_fp64": None if fp64 is None else v5 / fp64["value"],
                       "blowup_voxel_steps": s5.check(), "network": {k: net5.meta.get(k) for k in
                                                                    ("pairs", "tissue_pairs", "epochs",
                                                                     "macro_steps")}}
            s5.close()

        # ---- accuracy against the FP64 form (1.35M-voxel shell, a whole beat) ------
        accuracy = None
        if args.accuracy:
            accuracy = accuracy_leg(lq, net, stream, args.accuracy_ms, net5)
            if at_spec is not None and accuracy.get("surrogate_at_spec"):
                at_spec["accuracy"] = accuracy["surrogate_at_spec"]

        # ---- the other configurations of the reference's drivers -----------------
        configs = None
        if args.configs:
            configs = {"config1_oned_strand": config1_leg(lq), "config2_sheet2d": config2_leg(lq, net, stream)}

        # batched sweep leg: 4096 uneven single cells / strands (50-400 cells), own
        # parameters each, one persistent graph-captured launch (autotuned shape)
        sweep = None
        if args.sweep_beats > 0:
            insts, models, _ = lq.batch.sweep(n=4096, seed=2024, beats=args.sweep_beats)
            # ranks take contiguous shards of about equal work (no data collective)
            wk = [len(x.types) * round(x.t_stop / 0.02) for x in insts]
            lo, hi = replicas.shard_bounds(len(insts), rank, world, wk)
            mine = insts[lo:hi]
            for j, x in enumerate(mine):
                x.model = j
            bt = lq.Batch(mine, models[lo:hi], precision=lq.MIXED, max_beats=args.sweep_beats + 1,
                          stream=stream.cuda_stream)
            barrier()
            ms_local = bt.run()
            v_sw, ms_sw, work = replicas.aggregate_throughput(float(sum(wk[lo:hi])), ms_local)
            det = bt.detect()
            sweep = {"value": v_sw, "unit": UNIT, "instances": len(insts),
                     "cells": int(sum(len(x.types) for x in insts)), "beats": args.sweep_beats, "device_ms": ms_sw,
                     "launch": bt.config(), "scaling": "strong", "blowup_cell_steps": bt.num_bad(), "form": "mixed",
                     "ead_cells": int((det["ead"] > 0).sum()),
                     "error_vs_fp64": "per-instance APD90 and EAD flags against FP64 oracle instances on a seeded "
                                      "sub-sample: tests/test_gpu_sweep.py::test_sweep_at_stated_size_vs_fp64_oracle"}
            bt.close()
    finally:
        clk.__exit__(None, None, None)

    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline:
        r = run_cpu(w, 10_000, 1, seconds=15.0)
        r1 = run_cpu(w, 10_000, 1, seconds=10.0, threads=1, max_voxels=30_000)
        cpu = {"value": r["value"], "unit": UNIT, "cores": r["cores"], "kind": "port",
               "sample": f"{r['n']} tissue voxels (x-slab of the workload), {r['steps']} steps, FP64 oracle, "
                         f"OpenMP on {r['cores']} threads, {cpu_model_name()}",
               "single_thread": {"value": r1["value"], "cores": 1,
                                 "sample": f"{r1['n']} tissue voxels (x-slab), {r1['steps']} steps, 1 thread"}}
    clocks = clk.summary()
    # our kernels in the timed windows: per step the V-only substep, the plain
    # step over the listed voxels and the ghost/clock kernel; per macro step
    # the macro-step kernel; per 50 steps the two ECG kernels
    mac_timed = sum(p.get("macro_steps", 0) for p in per_phase.values())
    launches = 3 * ktot + mac_timed + 2 * (ktot // 50)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / ktot, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": w["desc"], "tissue_voxels": n,
                       "form": "FP32 + learned surrogate (FP32 gates/currents/diffusion, Kahan-compensated FP32 "
                               "concentrations; %g ms macro steps of a coarse TPORd step + BF16 tcgen05 MLP "
                               "correction where |dV/dt| <= %g mV/ms and not at a wave's foot (V < -40 mV rising "
                               "faster than %g mV/ms), plain 0.02 ms steps elsewhere)"
                               % (round(0.02 * net.nsub, 3), args.sur_dvdt_max, args.sur_foot_dvdt),
                       "surrogate_thresholds": dict(SUR_CFG),
                       "deviations_from_stated_config5": {
                           "macro_step_ms": [round(0.02 * net.nsub, 3), 0.1],
                           "dvdt_gate_mV_per_ms": [args.sur_dvdt_max, 1.0],
                           "training_pairs": ["paced single cells with the sweep's parameter ranges",
                                              "plain-integrator runs of configs 2 and 4"],
                           "stated_form_measured_in": "config5_at_spec"},
                       "timing": ("%d steps in each of the beat's phases %s, reached by untimed steps"
                                  % (args.steps, [p[0] for p in phases])) if phase_mode else
                                 "%d consecutive steps" % args.steps,
                       "dt_ms": 0.02, "electrodes": len(w["electrodes"]),
                       "l2": "inputs larger than L2 (state %.2f GB)" % (BYTES_MIXED * n / 1e9),
                       "parallelism": f"replicas x{world}",
                       "step_kernel_variant": {"min_ctas_per_sm": variant,
                                               "tuned_ms": [round(float(x), 4) for x in tune_ms[:3]]},
                       "substep_variant": {"chosen": sub_variant,
                                           "tuned_ms": dict(zip(("5", "6", "8", "105", "106", "108", "203", "204",
                                                                     "304", "305", "306"),
                                                                (round(float(x), 4) for x in sub_ms)))}},
            "windows": per_phase,
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "surrogate": surrogate, "mixed_form": mixed,
            "fp64_form": fp64, "config5_at_spec": at_spec, "accuracy": accuracy, "batched_sweep": sweep,
            "other_configs": configs, "gpu_launches": launches, "clocks": clocks, "blowup_voxel_steps": nbad}
    print(json.dumps(line), flush=True)


def e2e_leg(lq, torch, make_sim, stream, phases, k, world, variant, sub_variant, advance_to):
    """e2e through the C ABI with pinned host buffers, over the same windows
    as the headline: the initial state H2D once, then in every window k
    asynchronous steps each followed by a read-back of V to the host (the
    reference's host loop copies V back every step, GPU3D.cu:1802) on copy
    streams into a ring of pinned buffers, every copy complete inside the
    window, and the state D2H at the end.  The untimed steps between windows
    are outside the timed region."""
    sim = make_sim(lq.MIXED, True)
    n = sim.n
    sim.tune(variant)
    sim.substep_variant(sub_variant)
    st_host = torch.empty((n, 40), dtype=torch.float64, pin_memory=True).numpy()
    # host ring of 32 x 28 MB pinned buffers; before a buffer is reused the
    # host waits for the copy that last filled it (never for the newest one)
    ring = 32
    v_host = [torch.empty(n, dtype=torch.float32, pin_memory=True).numpy() for _ in range(ring)]
    last = [None] * ring            # the copy that last filled each host buffer
    sim.get_state(out=st_host)
    # setup, like creating the simulation: the first read-back allocates the
    # library's ring of device slots
    sim.get_v_async(v_host[0])
    sim.wait_v()
    nv = 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sim.set_state(st_host)
    t_h2d = time.perf_counter() - t0
    t_win = 0.0
    for _, tp in phases:
        if tp is not None:
            advance_to(sim, tp)
        sim.sync()
        t0 = time.perf_counter()
        for i in range(k):
            sim.step_async(1)
            j = nv % ring
            if last[j] is not None:
                sim.wait_v(last[j])                # the copy that last filled this buffer
            last[j] = sim.get_v_async(v_host[j])
            nv += 1
        sim.sync()
        sim.wait_v()
        t_win += time.perf_counter() - t0
    t0 = time.perf_counter()
    sim.get_state(out=st_host)
    t_d2h = time.perf_counter() - t0
    sim.close()
    ktot = k * len(phases)
    tot = t_h2d + t_win + t_d2h
    return {"value": world * n * ktot / tot, "unit": UNIT, "h2d_bytes_per_step": int(n * 320 / ktot),
            "d2h_bytes_per_step": int(n * 4 + n * 320 / ktot), "steps": ktot, "form": "FP32 + surrogate",
            "readback": "V of every voxel every step: gathered into 16 device slots, copied on 4 copy streams into a "
                        "ring of 32 pinned host buffers, each reused once its last copy is complete",
            "parts": {"state_h2d_ms": 1e3 * t_h2d, "state_d2h_ms": 1e3 * t_d2h,
                      "stepping_with_readback_ms": 1e3 * t_win,
                      "stepping_with_readback_value": world * n * ktot / t_win,
                      "state_bytes": int(n * 320)}}


def config1_leg(lq):
    """OneD.cc: 100 cells, 5 beats + 1 cycle (6 s), one persistent launch;
    launch-latency bound by construction (2.5e7 cell-steps).  Errors of the
    mixed form against the FP64 form over the first 2 beats (2000 ms):
    activation, APD90 per cell and beat, V records outside the upstroke,
    pseudo-ECG and conduction velocity."""
    out = {"workload": "OneD.cc strand, 100 cells, 6000 ms, V every 10 steps"}
    # FP64: one strand is one CTA on one SM at the FP64 rate; a 500 ms sample
    for name, prec, t_ms in (("fp64", lq.FP64, 500.0), ("mixed", lq.MIXED, 6000.0)):
        st = lq.OneDStrand(model="default", precision=prec, num_s1=5 if t_ms >= 6000.0 else 0, stop_time=t_ms)
        r = st.run()
        work = 100 * round(t_ms / 0.02)
        out[name] = {"device_ms": r["device_ms"], "cell_steps_per_s": work / (r["device_ms"] / 1e3),
                     "simulated_ms": t_ms}
        if prec == lq.MIXED:
            out[name]["cv_m_per_s"] = float(r["cv"])
    res = {}
    for name, prec in (("fp64", lq.FP64), ("mixed", lq.MIXED)):
        res[name] = lq.OneDStrand(model="default", precision=prec, num_s1=1, stop_time=2000.0).run()
    a, b = res["mixed"], res["fp64"]
    both = (a["t_act"] >= 0) & (b["t_act"] >= 0)
    bota = (a["apd90"] > 0) & (b["apd90"] > 0)
    # outside the upstroke: records more than 1 ms before / 5 ms after the
    # cell's activation in that cycle
    t = np.asarray(b["rec_t"])
    up = np.zeros(b["rec"].shape, bool)
    for j in range(b["t_act"].shape[1]):
        ta = b["t_act"][:, j]
        ok = ta >= 0
        up |= ok[None, :] & (t[:, None] >= ta[None, :] - 1.0) & (t[:, None] <= ta[None, :] + 5.0)
    dv = np.abs(a["rec"] - b["rec"])[~up]
    out["mixed_vs_fp64"] = {"window_ms": 2000.0, "activation_max_ms": float(np.abs(a["t_act"] - b["t_act"])[both].max()),
                            "apd90_max_ms": float(np.abs(a["apd90"] - b["apd90"])[bota].max()),
                            "apd90_compared": int(bota.sum()), "v_outside_upstroke_max_mV": float(dv.max()),
                            "ecg_max_rel": float(np.abs(a["ecg"] - b["ecg"]).max() / np.abs(b["ecg"]).max()),
                            "same_activations": bool(np.array_equal(a["t_act"] >= 0, b["t_act"] >= 0))}
    return out


def config2_leg(lq, net, stream):
    """The 600 x 600 sheet at 0.15 mm, S1 line at x = 0, S2 quadrant at a
    seeded coupling interval U[300, 360] ms, 2 s: mixed and FP32 + surrogate.
    Errors against the FP64 form on a 200 x 200 sheet with the same protocol
    over 1000 ms: the S1 wave's activation and APD90, the S2 wave's activation
    times, and V 50, 100, 200 ms after S2 and at 1000 ms."""
    import torch
    rng = np.random.default_rng(7)
    ci = float(rng.uniform(300.0, 360.0))
    m = lq.model("lqt1", gks_scale=0.5)
    out = {"workload": "2d-sheet 600x600 @0.15mm, S1 + S2 at %.1f ms, 2000 ms" % ci,
           "note": "the -104 pA/pF S2 over a whole quadrant for 3 ms lifts V to about 284 mV inside it (FP64 and "
                   "mixed alike; the reference's own S2, new_11.cu:1798-1803, is -104 pA/pF for 2 ms on a "
                   "100 x 150 patch); the blow-up count here is NaN/overflow only"}

    def make(n, sur, prec=lq.MIXED):
        sh = lq.geometry.sheet(n, n)
        sim = lq.Sim(sh.types, 0.15, precision=prec, model=m, stream=stream.cuda_stream, vmin_ok=-1e9, vmax_ok=1e9)
        sim.set_protocol(bcl=1000.0, s1_mask=sh.s1_mask, s1_start=0.0, s1_duration=2.0, s1_strength=-52.0,
                         s1_beats=1, s2_time=ci, s2_duration=3.0, s2_strength=-104.0, s2_mask=sh.s2_mask)
        if sur:
            sim.set_surrogate(net, **SUR_CFG)
        return sim

    nsteps = 100000
    for name, sur in (("mixed", False), ("surrogate", True)):
        sim = make(600, sur)
        sim.step(100)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(stream)
        sim.step(nsteps - 100)
        b.record(stream)
        torch.cuda.synchronize()
        ms = a.elapsed_time(b)
        out[name] = {"cell_steps_per_s": sim.n * (nsteps - 100) / (ms / 1e3), "device_ms": ms,
                     "blowup_voxel_steps": sim.check()}
        if sur:
            st = sim.surrogate_stats()
            out[name]["accepted_frac_of_voxel_macro_steps"] = st["accepted"] / max(1, st["macro_steps"] * sim.n)
        sim.close()
    # errors on the 200 x 200 sheet: the S1 wave by its detector (activation,
    # APD90); the S2 wave (the detector follows S1 cycles only) by its own
    # activation times -- V read back every step from S2 to S2 + 250 ms, the
    # first upward crossing of -30 mV at each voxel, as the detector times it
    # -- and by V 50, 100 and 200 ms after S2 and at 1000 ms
    res = {}
    t_mid = ci - 1.0
    snaps = (50.0, 100.0, 200.0)
    for name, sur, prec in (("fp64", False, lq.FP64), ("mixed", False, lq.MIXED), ("surrogate", True, lq.MIXED)):
        sim = make(200, sur, prec)
        sim.step(int(round(t_mid / 0.02)))
        d1 = sim.detect()
        sim.step(int(round(ci / 0.02)) - int(round(sim.time / 0.02)))
        vold = sim.get_v()
        act2 = np.full(sim.n, -1.0)
        vs = []
        for k in range(int(round(250.0 / 0.02))):
            t_pre = sim.time
            sim.step(1)
            v = sim.get_v()
            new = (vold < -30.0) & (v >= -30.0) & (act2 < 0)
            act2[new] = t_pre
            vold = v
            if any(abs(sim.time - (ci + dtm)) < 0.01 for dtm in snaps):
                vs.append(v.astype(np.float64))
        sim.step(int(round(1000.0 / 0.02)) - int(round(sim.time / 0.02)))
        vs.append(sim.get_v(as_double=True))
        res[name] = dict(act1=d1["t_act"], apd1=d1["apd90"], act2=act2, v=np.array(vs))
        s2m = lq.geometry.sheet(200, 200).s2_mask.reshape(-1)[sim.tissue_index()] > 0
        sim.close()
    ref = res["fp64"]
    err = {"workload": "2d-sheet 200x200 @0.15mm, same protocol, 1000 ms",
           "s2_wave_fp64": {"activated_outside_s2_quadrant": float((ref["act2"][~s2m] >= 0).mean()),
                            "last_activation_ms_after_s2": float(ref["act2"].max() - ci)}}
    for name in ("mixed", "surrogate"):
        d = res[name]
        k1 = (d["act1"] >= 0) & (ref["act1"] >= 0)
        ka = (d["apd1"] > 0) & (ref["apd1"] > 0)
        k2 = (d["act2"] >= 0) & (ref["act2"] >= 0)
        e2 = np.abs(d["act2"] - ref["act2"])[k2]
        dv = np.abs(d["v"] - ref["v"])
        err[name] = {"s1_activation_max_ms": float(np.abs(d["act1"] - ref["act1"])[k1].max()),
                     "s1_apd90_max_ms": float(np.abs(d["apd1"] - ref["apd1"])[ka].max()) if ka.any() else None,
                     "s2_wave_activation_max_ms": float(e2.max()) if e2.size else None,
                     "s2_wave_activation_mean_ms": float(e2.mean()) if e2.size else None,
                     "s2_wave_activation_p99_ms": float(np.percentile(e2, 99)) if e2.size else None,
                     "s2_wave_voxels": int(k2.sum()),
                     "s2_wave_voxels_only_here_or_only_fp64": int(((d["act2"] >= 0) != (ref["act2"] >= 0)).sum()),
                     "v_max_mV_at_s2_plus_50_100_200_and_1000ms": [round(float(x), 4) for x in dv.max(axis=1)],
                     "v_rms_mV_at_s2_plus_50_100_200_and_1000ms": [round(float(x), 5) for x in
                                                                  np.sqrt((dv ** 2).mean(axis=1))]}
    out["errors_vs_fp64"] = err
    return out


def accuracy_leg(lq, net, stream, t_ms, net5=None):
    """Errors of the FP32 forms against the FP64 form on the 1.35M-voxel shell
    (6 mm wall, the same construction and model as the 3D workload), S1 at
    t = 0, t_ms of the beat: APD90 and activation at every voxel, V outside
    the upstroke (snapshots every 10 ms, excluding 1 ms before to 5 ms after
    the voxel's activation), pseudo-ECG QT at six electrodes sampled every
    0.1 ms (T end: protocols.qt_from_ecg), and the device time and acceptance
    of each form.  The coarse step alone (no network) runs beside the
    surrogate: what the network gains is the ratio of their errors."""
    import torch
    from lqt1_gb300.protocols import qt_from_ecg
    w = build_workload("ventricle3d_small")
    nsteps = int(round(t_ms / 0.02))
    snap = 500
    out = {"workload": "3d-ventricle 170x170x220 @0.2mm, %d tissue voxels (6 mm wall), S1 at 0, %g ms"
                       % (int((w["types"] != 255).sum()), t_ms)}
    forms = [("fp64", lq.FP64, None, None), ("mixed", lq.MIXED, None, None),
             ("surrogate", lq.MIXED, net, dict(SUR_CFG)), ("coarse", lq.MIXED, net, dict(SUR_CFG, use_net=False))]
    if net5 is not None:
        forms.append(("surrogate_at_spec", lq.MIXED, net5, dict(SUR_AT_SPEC, nsub=net5.nsub)))
    ref = None
    for name, prec, mlp, cfg in forms:
        sim = lq.Sim(w["types"], 0.2, fibre=w["fibre"], precision=prec, model=workload_model(),
                     stream=stream.cuda_stream)
        sim.set_protocol(bcl=800.0, s1_mask=w["s1"], s1_start=0.0, s1_duration=2.0, s1_strength=-52.0, s1_beats=1)
        sim.set_electrodes(np.array(w["electrodes"]), every=5)
        if mlp is not None:
            sim.set_surrogate(mlp, **cfg)
        snaps, dev_ms = [], 0.0
        for _ in range(nsteps // snap):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            a.record(stream)
            sim.step(snap)
            b.record(stream)
            torch.cuda.synchronize()
            dev_ms += a.elapsed_time(b)
            snaps.append(sim.get_v())
        d = dict(det=sim.detect(), snaps=np.array(snaps), ecg=sim.ecg(), dev_ms=dev_ms, bad=sim.check(),
                 stats=sim.surrogate_stats() if mlp is not None else None)
        sim.close()
        qt = [qt_from_ecg(d["ecg"][1], d["ecg"][0][:, j], 0.15, 800.0)[0] for j in range(d["ecg"][0].shape[1])]
        if ref is None:
            ref = d
            ref["qt"] = qt
            t_act = d["det"]["t_act"]
            ts = snap * 0.02 * np.arange(1, len(d["snaps"]) + 1)
            calm = np.ones(d["snaps"].shape, bool)
            for i, t in enumerate(ts):
                calm[i] = ~((t >= t_act - 1.0) & (t <= t_act + 5.0))
            out["fp64"] = {"device_ms": dev_ms, "qt_ms": [round(x, 2) for x in qt],
                           "repolarised_by_ms": float((t_act + d["det"]["apd90"]).max())}
            continue
        e = d["det"]["apd90"] - ref["det"]["apd90"]
        both = (d["det"]["apd90"] > 0) & (ref["det"]["apd90"] > 0)
        act = (d["det"]["t_act"] >= 0) & (ref["det"]["t_act"] >= 0)
        dv = np.abs(d["snaps"] - ref["snaps"])[calm]
        r = {"apd90_max_ms": float(np.abs(e[both]).max()), "apd90_mean_ms": float(np.abs(e[both]).mean()),
             "apd90_bias_ms": float(e[both].mean()),
             "activation_max_ms": float(np.abs(d["det"]["t_act"] - ref["det"]["t_act"])[act].max()),
             "v_outside_upstroke_max_mV": float(dv.max()), "v_outside_upstroke_rms_mV": float(np.sqrt((dv ** 2).mean())),
             "qt_err_ms": [round(abs(a - b), 3) for a, b in zip(qt, ref["qt"])],
             "qt_err_max_ms": float(max(abs(a - b) for a, b in zip(qt, ref["qt"]))),
             "ecg_max_rel": float(np.abs(d["ecg"][0] - ref["ecg"][0]).max() / np.abs(ref["ecg"][0]).max()),
             "voxels_compared": int(both.sum()), "voxels_missing": int((~both).sum()), "device_ms": dev_ms,
             "cell_steps_per_s": len(e) * nsteps / (dev_ms / 1e3), "blowup_voxel_steps": d["bad"]}
        if d["stats"] is not None:
            st = d["stats"]
            r["accepted_frac_of_voxel_macro_steps"] = st["accepted"] / max(1, st["macro_steps"] * len(e))
        out[name] = r
        del d
    s, c = out["surrogate"], out["coarse"]
    out["network_gain"] = {
        "what": "coarse-step error / surrogate error (same macro steps and window, without the network)",
        "apd90_mean": c["apd90_mean_ms"] / max(s["apd90_mean_ms"], 1e-9),
        "apd90_max": c["apd90_max_ms"] / max(s["apd90_max_ms"], 1e-9),
        "v_outside_upstroke_rms": c["v_outside_upstroke_rms_mV"] / max(s["v_outside_upstroke_rms_mV"], 1e-9),
        "v_outside_upstroke_max": c["v_outside_upstroke_max_mV"] / max(s["v_outside_upstroke_max_mV"], 1e-9),
        "qt_err_max": c["qt_err_max_ms"] / max(s["qt_err_max_ms"], 1e-9),
        "speed_surrogate_over_coarse": s["cell_steps_per_s"] / c["cell_steps_per_s"]}
    return out


if __name__ == "__main__":
    main()
