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
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int, path: str | None = None):
        import tempfile
        self.device = device
        self.proc = None
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

    def summary(self):
        try:
            rows = [r.split(", ") for r in open(self.path).read().strip().splitlines() if r.strip()]
        except OSError:
            return None
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = max(float(r[2]) for r in rows if r[2].replace(".", "").isdigit())
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if len(r) > 5 + i and r[5 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows)}


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


def run_cpu(w, steps, warmup, seconds=None):
    from oracle import orc
    orc.build()
    sub, fib = cpu_sample(w)
    og = orc.Grid(sub, w["dx"], fibre=fib)
    m = orc.model(dict(dss_shift=0, fss_shift=0, pca_scale=2.0, gks_scale=0.5, gks_iso_scale=1.5, suprep_dose=0))
    st = orc.initial_state(-87.5, og.n)
    cores = os.cpu_count() or 1
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40000, help="timed steps (default: one 800 ms beat)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ventricle3d", choices=["ventricle3d", "ventricle3d_small", "sheet2d"])
    ap.add_argument("--prerun", type=int, default=0, help="untimed steps before the timed region (setup)")
    ap.add_argument("--weights", default=None, help="surrogate network file (default: the shipped network)")
    ap.add_argument("--clocks-csv", default=None, help="where to keep the raw nvidia-smi samples (default: temp dir)")
    ap.add_argument("--substep-variant", type=int, default=-1,
                    help="force the surrogate substep kernel (5/6/8 direct, 105/106/108 staged; -1 = autotune)")
    ap.add_argument("--sur-dvdt-max", type=float, default=1.5, help="surrogate eligibility: |dV/dt| bound, mV/ms")
    ap.add_argument("--sur-vstep-max", type=float, default=0.4, help="surrogate residual check: ionic dV per macro step")
    ap.add_argument("--fp64-steps", type=int, default=10)
    ap.add_argument("--mixed-steps", type=int, default=-1, help="steps of the plain mixed leg (-1 = --steps)")
    ap.add_argument("--no-accuracy", dest="accuracy", action="store_false")
    ap.add_argument("--no-configs", dest="configs", action="store_false",
                    help="skip the config 1 (OneD strand) and config 2 (2D sheet) legs")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sweep-beats", type=int, default=2,
                    help="beats of the 4096-instance batched sweep leg (0 = skip; 20 = the full sweep)")
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
    SUR_CFG.update(dvdt_max=args.sur_dvdt_max, vstep_max=args.sur_vstep_max)

    def make_sim(precision, surrogate):
        sim = lq.Sim(w["types"], w["dx"], fibre=w["fibre"], precision=precision, model=workload_model(),
                     detect=True, vmin_ok=-200.0, vmax_ok=200.0, stream=stream.cuda_stream)
        sim.set_protocol(bcl=w["bcl"], s1_mask=w["s1"], s1_start=0.0, s1_duration=2.0, s1_strength=-52.0,
                         s1_beats=3, s2_time=-1.0)
        sim.set_electrodes(np.array(w["electrodes"]), every=50)
        if surrogate:
            sim.set_surrogate(net, **SUR_CFG)
        return sim

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def timed(sim, steps, clk=None):
        """CUDA-event time of `steps` steps on the simulation's stream, max over ranks."""
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        sim.step(steps)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        _, ms, _ = replicas.aggregate_throughput(float(sim.n) * steps, e0.elapsed_time(e1))
        return ms

    # ---- headline: FP32 + surrogate form -----------------------------------
    sim = make_sim(lq.MIXED, True)
    n = sim.n
    sim.step(args.prerun)
    if args.substep_variant >= 0:
        sim.substep_variant(args.substep_variant)
    variant, tune_ms = sim.tune(-1)          # occupancy variant of the plain step kernel
    sub_variant, sub_ms = sim.substep_variant(-1, timings=True)   # and of the V-only substep
    sim.step(args.warmup)
    sim.surrogate_stats(reset=True)
    with ClockSampler(dev, args.clocks_csv) as clk:
        ms = timed(sim, args.steps)
    value = world * n * args.steps / (ms / 1e3)
    nbad = sim.check()
    sst = sim.surrogate_stats()
    ms_sub, ms_ghost_s, ms_sur = sim.profile(10)
    peaks = measured_peaks()
    peak = peaks.get("hbm_gbs")
    peak_kind = "measured" if peak else "fallback"
    peak = peak or 6800.0
    tpeak = peaks.get("bf16_tflops_sustained") or peaks.get("bf16_tflops") or 1700.0
    # dominant kernel of the surrogate form: the macro-step kernel (one launch
    # per macro step), algorithmic bytes and tensor FLOPs per voxel per launch
    ach_sur = BYTES_SUR_MACRO * n / (ms_sur / 1e3) / 1e9
    roof = {"bound": "hbm", "achieved": ach_sur, "peak": peak, "unit": "GB/s", "frac": ach_sur / peak,
            "traffic": traffic_summary("k_sur_grid_ventricle3d.json"), "kernel": "k_sur_grid", "kernel_ms": ms_sur,
            "bytes_per_voxel_launch": BYTES_SUR_MACRO, "peak_source": peak_kind,
            "tensor": {"achieved_tflops": FLOP_SUR_MACRO * n / (ms_sur / 1e3) / 1e12, "peak_tflops": tpeak,
                       "frac": FLOP_SUR_MACRO * n / (ms_sur / 1e3) / 1e12 / tpeak,
                       "flop_per_voxel_launch": FLOP_SUR_MACRO},
            "substep": {"kernels": "k_sur_substep + k_grid_step over the plain-voxel list", "ms": ms_sub,
                        "ghost_ms": ms_ghost_s}}
    surrogate = {"macro_steps": sst["macro_steps"], "voxel_offers": sst["offered"], "accepted": sst["accepted"],
                 "accepted_frac_of_voxel_macro_steps": sst["accepted"] / max(1, sst["macro_steps"] * n),
                 "wait_timeouts": sst["wait_timeouts"], "network": {k: net.meta.get(k) for k in
                                                                   ("pairs", "unique_pairs", "epochs",
                                                                    "oversample_phase3", "gen_and_train_s")}}

    # e2e through the C ABI with pinned host buffers: initial state H2D, then
    # every step lqt_sim_step_async + a read-back of V to the host (the reference's
    # host loop copies V back every step, GPU3D.cu:1802) -- asynchronous, on a
    # copy stream that overlaps the next step, all copies complete inside the
    # timed region -- and the final state D2H.
    st_host = torch.empty((n, 40), dtype=torch.float64, pin_memory=True).numpy()
    # pinned host buffers; a buffer is reused after a wait, and a wait drains
    # every copy in flight (the GPU idles while the host waits on the newest
    # one), so the ring is deep: 32 x 28 MB, one wait per 32 steps
    ring = 32
    v_host = [torch.empty(n, dtype=torch.float32, pin_memory=True).numpy() for _ in range(ring)]
    sim.get_state(out=st_host)
    k_e2e = max(10, args.steps)    # the same number of steps (a whole beat by default) as the headline
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sim.set_state(st_host)
    for i in range(k_e2e):
        sim.step_async(1)
        if i % ring == 0 and i > 0:
            sim.wait_v()
        sim.get_v_async(v_host[i % ring])
    sim.sync()
    sim.wait_v()
    sim.get_state(out=st_host)
    t_e2e = time.perf_counter() - t0
    e2e = {"value": world * n * k_e2e / t_e2e, "unit": UNIT, "h2d_bytes_per_step": int(n * 320 / k_e2e),
           "d2h_bytes_per_step": int(n * 4 + n * 320 / k_e2e), "steps": k_e2e, "form": "FP32 + surrogate",
           "readback": "V of every voxel every step, asynchronous on a copy stream"}
    sim.close()

    # ---- plain mixed form over the same steps ------------------------------
    mixed = None
    if args.mixed_steps != 0:
        ksteps = args.steps if args.mixed_steps < 0 else args.mixed_steps
        sm = make_sim(lq.MIXED, False)
        sm.step(args.prerun)
        variant_m, tune_m = sm.tune(-1)
        sm.step(args.warmup)
        ms_m = timed(sm, ksteps)
        ms_step, ms_ghost, _ = sm.profile(20)
        ach = BYTES_MIXED * n / (ms_step / 1e3) / 1e9
        mixed = {"value": world * n * ksteps / (ms_m / 1e3), "unit": UNIT, "steps": ksteps,
                 "surrogate_over_mixed": value / (world * n * ksteps / (ms_m / 1e3)),
                 "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                              "traffic": traffic_summary("k_grid_step_ventricle3d.json"),
                              "kernel": "k_grid_step<float,3>", "kernel_ms": ms_step,
                              "bytes_per_cell_step": BYTES_MIXED, "peak_source": peak_kind},
                 "step_kernel_variant": {"min_ctas_per_sm": variant_m,
                                         "tuned_ms": [round(float(x), 4) for x in tune_m[:3]]},
                 "blowup_voxel_steps": sm.check()}
        sm.close()

    # ---- plain FP64 form on the same state ----------------------------------
    fp64 = None
    if args.fp64_steps > 0:
        s64 = make_sim(lq.FP64, False)
        s64.set_state(st_host)
        s64.step(2)
        ms64t = timed(s64, args.fp64_steps)
        v64 = n * args.fp64_steps / (ms64t / 1e3)
        ms64, _, _ = s64.profile(2)
        fp64 = {"value": v64 * world, "unit": UNIT, "steps": args.fp64_steps, "kernel_ms": ms64,
                "achieved_gbs": BYTES_FP64 * n / (ms64 / 1e3) / 1e9, "surrogate_over_fp64": value / (v64 * world)}
        s64.close()

    # ---- accuracy of the surrogate form against the FP64 form ----------------
    accuracy = None
    if args.accuracy:
        accuracy = accuracy_leg(lq, net, stream)

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
        sweep = {"value": v_sw, "unit": UNIT, "instances": len(insts), "cells": int(sum(len(x.types) for x in insts)),
                 "beats": args.sweep_beats, "device_ms": ms_sw, "launch": bt.config(), "scaling": "strong",
                 "blowup_cell_steps": bt.num_bad(), "form": "mixed"}
        bt.close()

    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline:
        r = run_cpu(w, 10_000, 1, seconds=15.0)
        cpu = {"value": r["value"], "unit": UNIT, "cores": r["cores"], "kind": "port",
               "sample": f"{r['n']} tissue voxels (x-slab of the workload), {r['steps']} steps, FP64 oracle, "
                         f"OpenMP on {r['cores']} threads, {cpu_model_name()}"}
    clocks = clk.summary()
    # our kernels in the timed region: per step the V-only substep, the plain
    # step over the listed voxels and the ghost/clock kernel; per macro step
    # (net.nsub steps) the macro-step kernel; per 50 steps the two ECG kernels
    launches = 3 * args.steps + sst["macro_steps"] + 2 * (args.steps // 50)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": w["desc"], "tissue_voxels": n,
                       "form": "FP32 + learned surrogate (FP32 gates/currents/diffusion, Kahan-compensated FP32 "
                               "concentrations; %g ms macro steps of a coarse TPORd step + BF16 tcgen05 MLP "
                               "correction where |dV/dt| <= %g mV/ms, plain 0.02 ms steps elsewhere)"
                               % (round(0.02 * net.nsub, 3), args.sur_dvdt_max),
                       "surrogate_thresholds": dict(SUR_CFG),
                       "dt_ms": 0.02, "t_ms": [round((args.prerun + args.warmup + 15) * 0.02, 2),
                                               round((args.prerun + args.warmup + 15 + args.steps) * 0.02, 2)],
                       "electrodes": len(w["electrodes"]),
                       "l2": "inputs larger than L2 (state %.2f GB)" % (BYTES_MIXED * n / 1e9),
                       "parallelism": f"replicas x{world}",
                       "step_kernel_variant": {"min_ctas_per_sm": variant,
                                               "tuned_ms": [round(float(x), 4) for x in tune_ms[:3]]},
                       "substep_variant": {"chosen": sub_variant,
                                           "tuned_ms": dict(zip(("5", "6", "8", "105", "106", "108"),
                                                                (round(float(x), 4) for x in sub_ms)))}},
            "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "surrogate": surrogate, "mixed_form": mixed,
            "fp64_form": fp64, "accuracy": accuracy, "batched_sweep": sweep, "other_configs": configs,
            "gpu_launches": launches,
            "clocks": clocks, "blowup_voxel_steps": nbad}
    print(json.dumps(line), flush=True)


def config1_leg(lq):
    """OneD.cc: 100 cells, 5 beats + 1 cycle (6 s), one persistent launch;
    launch-latency bound by construction (2.5e7 cell-steps)."""
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
    return out


def config2_leg(lq, net, stream):
    """The 600 x 600 sheet at 0.15 mm, S1 line at x = 0, S2 quadrant at a
    seeded coupling interval U[300, 360] ms, 2 s: mixed and FP32 + surrogate."""
    import torch
    rng = np.random.default_rng(7)
    ci = float(rng.uniform(300.0, 360.0))
    sh = lq.geometry.sheet(600, 600)
    m = lq.model("lqt1", gks_scale=0.5)
    out = {"workload": "2d-sheet 600x600 @0.15mm, S1 + S2 at %.1f ms, 2000 ms" % ci,
           "note": "the -104 pA/pF S2 over a whole quadrant lifts V to about 284 mV inside it (FP64 and mixed "
                   "alike); the blow-up count here is NaN/overflow only"}
    nsteps = 100000
    for name, sur in (("mixed", False), ("surrogate", True)):
        sim = lq.Sim(sh.types, 0.15, precision=lq.MIXED, model=m, stream=stream.cuda_stream, vmin_ok=-1e9,
                     vmax_ok=1e9)
        sim.set_protocol(bcl=1000.0, s1_mask=sh.s1_mask, s1_start=0.0, s1_duration=2.0, s1_strength=-52.0,
                         s1_beats=1, s2_time=ci, s2_duration=3.0, s2_strength=-104.0, s2_mask=sh.s2_mask)
        if sur:
            sim.set_surrogate(net, **SUR_CFG)
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
    return out


def accuracy_leg(lq, net, stream):
    """APD90 and activation-time error of the surrogate form (and of the plain
    mixed form) against the FP64 form: 100k-voxel ventricle shell of the same
    construction, same model, one S1 beat (790 ms)."""
    v = lq.geometry.ventricle(nx=64, ny=64, nz=84, a_out=5.8, c_out=14.0, wall=3.0, z_base=15.5, island_radius=2.0,
                              stim_radius=1.2)
    nsteps = 39500
    out = {"workload": "3d-ventricle 64x64x84 @0.2mm, %d tissue voxels, 1 beat" % int((v.types != 255).sum())}
    res = {}
    for name, prec, sur in (("fp64", lq.FP64, False), ("mixed", lq.MIXED, False), ("surrogate", lq.MIXED, True)):
        sim = lq.Sim(v.types, 0.2, fibre=v.fibre, precision=prec, model=workload_model(), stream=stream.cuda_stream)
        sim.set_protocol(bcl=800.0, s1_mask=v.s1_mask, s1_start=0.0, s1_duration=2.0, s1_strength=-52.0,
                         s1_beats=1)
        if sur:
            sim.set_surrogate(net, **SUR_CFG)
        sim.step(nsteps)
        res[name] = sim.detect()
        sim.close()
    ref = res["fp64"]
    for name in ("mixed", "surrogate"):
        d = res[name]
        both = (d["apd90"] > 0) & (ref["apd90"] > 0)
        ea = np.abs(d["apd90"] - ref["apd90"])[both]
        act = (d["t_act"] >= 0) & (ref["t_act"] >= 0)
        et = np.abs(d["t_act"] - ref["t_act"])[act]
        out[name] = {"apd90_max_ms": float(ea.max()), "apd90_mean_ms": float(ea.mean()),
                     "activation_max_ms": float(et.max()), "voxels_compared": int(both.sum()),
                     "voxels_missing": int((~both).sum())}
    return out


if __name__ == "__main__":
    main()
