#!/usr/bin/env python3
"""Benchmark: particle-steps/s of LF_DEM's per-timestep hydrodynamic core on GB300.

Workload (the metric's configuration): N = 4096 bidisperse spheres (radii 1 and
1.4, equal volume shares), volume fraction 0.56, stress control sigma = 10
critical-load units (friction_model 2), mu = 1, lubrication lambda = 1e-3,
lub_max_gap 0.5, kn = 1e4, kt = 0.5 kn, seeded synthetic packing (there is no
public dataset).  One step = one full predictor-corrector time step
(2 assemblies, 2 factorisations, 2 x 4 right-hand-side solves, stresslets and
shear-rate solve each half step).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
  python bench.py --workload cfg3            (the 2D monolayer, N=8192)
  python bench.py --workload sweep|serve     (the batched and serving forms)

value        : particle-steps/s of the FP32 + FP64-refinement form, device time
               (CUDA events on the engine's stream), state resident in HBM
fp64_value   : the same for the plain FP64 form
e2e          : through the C ABI with host buffers: create from host arrays
               (H2D), K steps each followed by a D2H read of positions,
               velocities and the stress tensor
cpu_baseline : the CPU oracle (C restatement, OpenMP) on three steps of the
               same workload on this machine's host cores, plus one step on
               one thread; its first step is the reference of the accuracy
               figures (fp32_vs_oracle, fp64_vs_oracle: velocities, angular
               velocities, contact forces, stress, viscosity, N1, N2)
"""
from __future__ import annotations

import argparse
import datetime
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

N_PART = 4096
VF = 0.56
SIGMA_CL = 10.0
METRIC = "particle-steps/s at N=4096 phi=0.56, FP32+refine vs FP64 direct; p50/p99 latency"


def workload_params():
    return dict(kn=1e4, kt=5e3, mu_static=1.0, mu_dynamic=1.0, friction_model=2, critical_load=1.0,
                repulsion_on=0, repulsion=0.0, repulsive_length=0.05, repulsive_max_length=-1.0,
                lubrication_model=2, lub_reduce_parameter=1e-3, lub_max_gap=0.5, interaction_range=-1.0,
                sd_coeff=1.0, contact_relaxation_time=1e-3, contact_relaxation_time_tan=-1.0, disp_max=1e-3,
                dt=1e-4, dt_max=-1.0, dt_min=-1.0, fixed_dt=0, integration_method=1, control=1,
                shear_rate=0.0, target_stress=SIGMA_CL / 6 / np.pi, Ehat=(0, 0, 0.5, 0, 0, 0),
                Ohat=(0, 0.5, 0), init_strain_shear_rate_limit=0.0, init_shear_rate_limit=999.0, ft_max=0.0)


def config(world):
    return {"workload": f"3D stress-controlled critical-load model: N={N_PART} bidisperse 1:1.4, phi={VF}, "
                        f"sigma={SIGMA_CL:g}cl, mu=1, lambda=1e-3, kn=1e4, predictor-corrector",
            "n_particles": N_PART, "volume_fraction": VF, "control": "stress 10cl",
            "parallelism": f"replicas x{world}" if world > 1 else "single suspension",
            "l2": "inputs larger than L2 (fronts 0.8-1.7 GB per factorisation)"}


class ClockSampler:
    """nvidia-smi clocks every 20 ms; stop(window) keeps the samples whose own
    timestamps fall inside the timed region (host wall-clock interval)."""
    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self, window=None):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.05)   # the sample after the window's end
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 10:
                continue
            try:
                ts = datetime.datetime.strptime(f[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                rows.append((ts, float(f[2]), float(f[3]), f[6:10]))
            except ValueError:
                continue
        inside = [r for r in rows if window and window[0] <= r[0] <= window[1]]
        use = inside if inside else rows
        sm = [r[1] for r in use]
        smax = [r[2] for r in use]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in use:
            for nm, v in zip(names, r[3]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm),
                "window": "timed region" if inside else "whole run (no sample inside the timed region)"}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), d.get("bf16_tflops_sustained", 1700.0), \
            "measured"
    except (OSError, ValueError):
        return 6800.0, 1900.0, 1700.0, "fallback"


def run_engine(E, packing, precision, steps, warmup, device):
    params = workload_params()
    g = E.Sim(params, packing.position, packing.radius, packing.lx, packing.ly, packing.lz,
              precision=precision, device=device)
    g.run(warmup)
    g.clear_step_times()
    t0 = time.time()
    g.run(steps)
    t1 = time.time()
    ms, kernels = g.step_times()
    timing = g.timing()
    sc = g.scalars()
    g.close()
    run_engine.window = (t0, t1)
    return ms, kernels, timing, sc


def _step_record(part, sc, pairs):
    return {"vel": part["vel"], "ang": part["ang"], "total_stress": sc["total_stress"],
            "viscosity": sc["viscosity"], "N1": sc["N1"], "N2": sc["N2"],
            "keys": np.stack([pairs["p0"], pairs["p1"]], 1), "contact_force": np.asarray(pairs["f_spring_total"])}


def _errors(a, b):
    """Largest relative differences of record a against record b (each
    relative to the largest magnitude of b's quantity)."""
    rel = lambda x, y: float(np.abs(np.asarray(x) - np.asarray(y)).max() / max(np.abs(np.asarray(y)).max(), 1e-300))
    out = {k: rel(a[k], b[k]) for k in ("vel", "ang", "total_stress", "viscosity", "N1", "N2")}
    out["contact_force"] = rel(a["contact_force"], b["contact_force"]) if np.array_equal(a["keys"], b["keys"]) \
        else None
    out["pair_list_identical"] = bool(np.array_equal(a["keys"], b["keys"]))
    return out


def rebuild_cost(E, packing, device, steps=12, skin=0.001):
    """The host cost of one pattern change at this workload: a short run with
    a pair-superset skin so thin that the superset goes stale nearly every
    step, so that each rebuild (candidate pairs, symbolic analysis, upload,
    graph capture) is timed; the default skin changes the pattern far less
    often (pattern_changes)."""
    g = E.Sim(workload_params(), packing.position, packing.radius, packing.lx, packing.ly, packing.lz,
              precision=E.PREC_FP32_REFINE, device=device, skin=skin)
    g.run(2)
    g.clear_step_times()
    g.run(steps)
    tim = g.timing()
    g.close()
    r = tim["rebuilds"]
    return {"steps": steps, "skin": skin, "rebuilds": r,
            "rebuild_host_ms_mean": tim["rebuild_ms"] / r if r else None}


def pattern_changes(E, packing, device, steps):
    """A longer run of the FP32 + refinement form from the packing, long
    enough for the pair superset to run out of skin: how often the pattern of
    R_FU changes (superset rebuild + symbolic analysis, cholmod_analyze's
    counterpart), what one rebuild costs on the host (including the capture
    of the new factorisation and solve graphs), and the throughput with those
    rebuilds folded in: particle-steps / host wall-clock time of the whole
    run."""
    params = workload_params()
    g = E.Sim(params, packing.position, packing.radius, packing.lx, packing.ly, packing.lz,
              precision=E.PREC_FP32_REFINE, device=device)
    g.run(3)
    g.clear_step_times()
    s0 = g.scalars()["strain"]
    t0 = time.perf_counter()
    g.run(steps)
    wall = time.perf_counter() - t0
    ms, _ = g.step_times()
    tim = g.timing()
    sc = g.scalars()
    g.close()
    r = tim["rebuilds"]
    return {"steps": steps, "strain_covered": float(sc["strain"] - s0), "rebuilds": r,
            "steps_per_rebuild": steps / r if r else None,
            "rebuild_host_ms_total": tim["rebuild_ms"], "rebuild_host_ms_mean": tim["rebuild_ms"] / r if r else None,
            "device_ms_per_step": float(np.mean(ms)), "wall_ms_per_step": 1e3 * wall / steps,
            "value_amortised": N_PART * steps / wall, "unit": "particle-steps/s",
            "note": "host wall clock over the whole run, rebuilds (candidate pairs, symbolic analysis, "
                    "upload, graph capture) included"}


def accuracy(E, packing, device, oracle_ref=None):
    """One predictor-corrector step with stresses from the packing, in the
    FP32 + refinement and the FP64 forms: largest relative differences of the
    velocities, angular velocities, contact forces, total stress, viscosity,
    N1 and N2 against the CPU oracle's step from the same state (when given)
    and between the two forms, with the refinement's counts."""
    params = workload_params()
    rec = {}
    for prec in (E.PREC_FP64, E.PREC_FP32_REFINE):
        g = E.Sim(params, packing.position, packing.radius, packing.lx, packing.ly, packing.lz,
                  precision=prec, device=device)
        g.step(calc_stress=True)
        rec[prec] = (_step_record(g.particles(), g.scalars(), g.pairs()), g.scalars())
        g.close()
    (r64, _), (r32, s32) = rec[E.PREC_FP64], rec[E.PREC_FP32_REFINE]
    out = {"fp32_vs_fp64": dict(_errors(r32, r64), refine_iters=int(s32["last_refine_iters"]),
                                refine_residual=float(s32["last_refine_residual"]),
                                note="one predictor-corrector step from the same state, FP32 factor + FP64 "
                                     "refinement vs FP64 factor")}
    if oracle_ref is not None:
        out["fp32_vs_oracle"] = dict(_errors(r32, oracle_ref),
                                     note="one step from the packing against the CPU oracle (FP64)")
        out["fp64_vs_oracle"] = dict(_errors(r64, oracle_ref),
                                     note="one step from the packing against the CPU oracle (FP64)")
    return out


def run_e2e(E, packing, precision, steps, device):
    """Create from host arrays, K steps, each followed by a D2H read of the state."""
    import ctypes as C
    params = workload_params()
    pos = np.ascontiguousarray(packing.position)
    rad = np.ascontiguousarray(packing.radius)
    t0 = time.perf_counter()
    g = E.Sim(params, pos, rad, packing.lx, packing.ly, packing.lz, precision=precision, device=device)
    t_created = time.perf_counter()
    L = E.load()
    outp = np.zeros(3 * len(rad))
    outv = np.zeros(3 * len(rad))
    for _ in range(steps):
        g.step()
        L.lfg_sim_get_particles(g.h, outp.ctypes.data_as(C.c_void_p), outv.ctypes.data_as(C.c_void_p),
                                None, None, None)
        g.scalars()
    t1 = time.perf_counter()
    g.close()
    n = len(rad)
    return {"value": n * steps / (t1 - t0), "unit": "particle-steps/s",
            "h2d_bytes_per_step": int((pos.nbytes + rad.nbytes) / steps),
            # positions and velocities, and lfg_sim_get_scalars: the clock (240 B), the
            # per-component stress totals (11 x 6 doubles) and the interaction counts
            "d2h_bytes_per_step": int(outp.nbytes + outv.nbytes + 240 + 11 * 6 * 8 + 16),
            "create_ms": 1e3 * (t_created - t0), "steps_ms": 1e3 * (t1 - t_created),
            "note": "includes creation (H2D of the configuration, symbolic analysis, graph capture)"}


def cpu_baseline(packing, nsteps=3, one_thread=True):
    """The CPU oracle on this machine's host cores: nsteps predictor-corrector
    steps of the workload from the packing with all OpenMP threads (the first
    one with stresses; its result is the accuracy reference), then one step on
    one thread.  Returns (baseline record, the first step's result)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    pyoracle.build()
    cores = pyoracle.num_threads()
    method = _cpu_factorisation(pyoracle)
    o = pyoracle.OracleSim(workload_params(), packing.position, packing.radius, packing.lx, packing.ly,
                           packing.lz)
    o.first_time()
    t0 = time.perf_counter()
    o.step(calc_stress=True)
    t1 = time.perf_counter()
    ref = _step_record(o.particles(), o.scalars(), o.pairs())
    for _ in range(nsteps - 1):
        o.step()
    t2 = time.perf_counter()
    fs = pyoracle.factor_stats(o)
    steps_s = [t1 - t0, (t2 - t1) / max(nsteps - 1, 1)]
    rec = {"value": N_PART * nsteps / (t2 - t0), "unit": "particle-steps/s", "cores": cores, "kind": "port",
           "sample": f"{nsteps} predictor-corrector steps of the N={N_PART} workload from the packing, "
                     f"{t2 - t0:.1f} s; first step with stresses {steps_s[0]:.2f} s",
           "factorisation": method,
           "factor_flops_per_factorisation": fs["factor_flops"],
           "factor_gflops": fs["factor_flops"] * fs["factorisations"] / max(fs["factor_s"], 1e-12) / 1e9,
           "factor_s_per_factorisation": fs["factor_s"] / max(fs["factorisations"], 1),
           "analyze_s_per_factorisation": fs["analyze_s"] / max(fs["factorisations"], 1),
           "cpu": _cpu_model()}
    del o
    if one_thread:
        pyoracle.set_num_threads(1)
        if pyoracle.lib().lfo_blas_ready():
            pyoracle.use_blas(threads=1)   # the BLAS library's threads too
        o1 = pyoracle.OracleSim(workload_params(), packing.position, packing.radius, packing.lx, packing.ly,
                                packing.lz)
        o1.first_time()
        t0 = time.perf_counter()
        o1.step()
        t1 = time.perf_counter()
        fs1 = pyoracle.factor_stats(o1)
        rec["one_thread"] = {"value": N_PART / (t1 - t0), "unit": "particle-steps/s", "cores": 1,
                             "sample": f"1 predictor-corrector step, {t1 - t0:.1f} s",
                             "factor_gflops": fs1["factor_flops"] * fs1["factorisations"] /
                             max(fs1["factor_s"], 1e-12) / 1e9}
        del o1
        pyoracle.set_num_threads(cores)
        if pyoracle.lib().lfo_blas_ready():
            pyoracle.use_blas(threads=cores)
    return rec, ref


ARM_PARTS = {"0xd4f": "Arm Neoverse V2", "0xd40": "Arm Neoverse V1", "0xd0c": "Arm Neoverse N1",
             "0xd49": "Arm Neoverse N2"}


def _cpu_factorisation(pyoracle):
    """The CPU oracle's factorisation for the baseline: supernodal with dense
    BLAS-3 kernels (CHOLMOD's method) when scipy's BLAS/LAPACK is present."""
    if pyoracle.use_blas():
        return ("FP64 supernodal multifrontal Cholesky (minimum-degree ordering on the 6x6 blocks, relaxed "
                "supernodes), dense kernels dpotrf/dtrsm/dsyrk/dgemm from scipy's OpenBLAS, small fronts in "
                "parallel with OpenMP")
    return "FP64 block Cholesky (minimum degree on 6x6 blocks, right-looking, OpenMP trailing update)"


def _cpu_model():
    try:
        with open("/proc/cpuinfo") as f:
            txt = f.read()
        for key in ("model name", "Model name", "CPU part"):
            for ln in txt.splitlines():
                if ln.startswith(key):
                    v = ln.split(":", 1)[1].strip()
                    return f"{ARM_PARTS.get(v, v)} ({os.cpu_count()} logical CPUs)"
    except OSError:
        pass
    import platform
    return f"{platform.machine()} ({os.cpu_count()} logical CPUs)"


def dist_setup(backend="nccl"):
    """Ranks from the torchrun environment.  Each rank runs an independent
    replica (one suspension per GPU); the process group only carries the
    barrier and the max-over-ranks of the timed region."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
        return world, rank, local, dist, torch
    return world, rank, local, None, None


def max_over_ranks(value, dist, torch, device):
    """The slowest rank's time (weak scaling: every rank times its own replica)."""
    if dist is None:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(n_particles, steps, world, slowest_s):
    """Whole-job particle-steps/s: all ranks' particle-steps over the slowest rank's time."""
    return n_particles * steps * world / slowest_s


def reference_arm(args):
    world, rank, local, dist, torch = dist_setup()
    if rank != 0:
        return
    from lf_dem_gb300 import packing as PK
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    pyoracle.build()
    method = _cpu_factorisation(pyoracle)
    p = PK.generate(N_PART, VF, seed=2000)
    o = pyoracle.OracleSim(workload_params(), p.position, p.radius, p.lx, p.ly, p.lz)
    o.first_time()
    for _ in range(args.warmup):
        o.step()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        o.step()
        times.append(time.perf_counter() - t0)
    tot = sum(times)
    val = N_PART * args.steps / tot
    fs = pyoracle.factor_stats(o)
    line = {"metric": METRIC, "value": val, "unit": "particle-steps/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": config(1),
            "p50_ms": 1e3 * float(np.percentile(times, 50)), "p99_ms": 1e3 * float(np.percentile(times, 99)),
            "cpu_baseline": {"value": val, "unit": "particle-steps/s", "cores": pyoracle.num_threads(),
                             "kind": "port",
                             "sample": f"{args.steps} full steps of the N={N_PART} workload on the CPU oracle "
                                       "(C restatement of LF_DEM's step; reference C++ + CHOLMOD cannot be "
                                       "built on this host)",
                             "factorisation": method,
                             "factor_flops_per_factorisation": fs["factor_flops"],
                             "factor_gflops": fs["factor_flops"] * fs["factorisations"] /
                             max(fs["factor_s"], 1e-12) / 1e9, "cpu": _cpu_model()},
            "e2e": {"value": val, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _gen_packing(args):
    from lf_dem_gb300 import packing as PK
    n, vf, seed = args
    return PK.generate(n, vf, seed=seed)


def gen_packings(specs):
    """Seeded packings, generated in a spawn pool before any GPU call."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Pool(min(16, os.cpu_count() or 1)) as pool:
        return pool.map(_gen_packing, specs)


def rate_params(rate):
    p = workload_params()
    p.update(friction_model=1, critical_load=0.0, repulsion_on=1, repulsion=1.0, control=0, shear_rate=rate,
             target_stress=0.0)
    return p


def stress_params(sigma_cl):
    p = workload_params()
    p.update(target_stress=sigma_cl / 6 / np.pi)
    return p


def bench_sweep(args):
    """Batched rheology sweep: 64 independent 3D suspensions, N ~ U[256, 2048],
    phi ~ U[0.45, 0.58], rate control with shear rates log-spaced 1e-2..1e2
    (repulsive-force units), bidisperse 1:1.4, FP32 + refinement.  Three ways
    to advance them K steps each, aggregate particle-steps/s over host wall
    time: fused (one joint factorisation and solve per half step for all of
    them, each half step a captured CUDA graph; leaf size picked by the
    autotuner on the fused step), concurrent (each on its own stream, 16 host
    workers) and one host thread (one after another)."""
    rng = np.random.default_rng(4000)
    m = args.count or 64
    ns = rng.integers(256, 2049, size=m)
    vfs = rng.uniform(0.45, 0.58, size=m)
    rates = np.logspace(-2, 2, m)
    packs = gen_packings([(int(n), float(v), 4000 + k) for k, (n, v) in enumerate(zip(ns, vfs))])
    import lf_dem_gb300 as E
    from lf_dem_gb300 import build as B
    B.build()
    E.load()
    out = {}
    modes = (("fused", 0), ("concurrent", 16), ("one_thread", 1))
    if getattr(args, "sweep_modes", None):
        modes = tuple(m for m in modes if m[0] in args.sweep_modes)
    for label, threads in modes:
        if label == "fused":
            b = E.Batch(fused=True, precision=E.PREC_FP32_REFINE)
        else:
            b = E.Batch(nthreads=threads)
        t0 = time.perf_counter()
        for p, r in zip(packs, rates):
            b.add(rate_params(float(r)), p.position, p.radius, p.lx, p.ly, p.lz, precision=E.PREC_FP32_REFINE)
        create_s = time.perf_counter() - t0
        rec = {"create_s": create_s}
        if label != "one_thread":
            t0 = time.perf_counter()
            b.autotune((8, 16, 32), steps=1)
            rec["autotune_s"] = time.perf_counter() - t0
            rec["tuned_leaf"] = {str(n): b.tuned_leaf(n, 1) for n in (256, 512, 1024, 2048)}
        b.run(args.warmup)
        k0 = b.stats()["kernels"]
        t0 = time.perf_counter()
        b.run(args.steps)
        wall = time.perf_counter() - t0
        st = b.stats()
        rec.update({"particle_steps_per_s": float(ns.sum()) * args.steps / wall, "wall_s": wall,
                    "host_threads": threads if label != "fused" else 1,
                    "kernels_per_batch_step": (st["kernels"] - k0) / args.steps})
        if label == "fused":
            rec.update({"joint_factor_gflop": st["factor_flops"] / 1e9, "joint_analyses": st["joint_analyses"],
                        "refine_iters": st["last_refine_iters"]})
        out[label] = rec
        b.close()
    line = {"metric": "aggregate particle-steps/s, batched sweep", "workload": "sweep",
            "value": out["fused"]["particle_steps_per_s"], "unit": "particle-steps/s",
            "steps": args.steps, "warmup": args.warmup, "dtype": "f32+f64refine", "data": "synthetic",
            "config": {"suspensions": m, "n_range": [256, 2048], "phi_range": [0.45, 0.58],
                       "shear_rates": "log-spaced 1e-2..1e2 (repulsive-force units)", "control": "rate",
                       "total_particles": int(ns.sum()),
                       "note": "fixed step count per suspension instead of 2 strain units; host wall time"},
            **out}
    for other in ("concurrent", "one_thread"):
        if other in out:
            line[f"fused_vs_{other}"] = out["fused"]["particle_steps_per_s"] / out[other]["particle_steps_per_s"]
    return line


def monolayer_params():
    """2D monolayer: rate control 1r (repulsive-force units), kn = 1e4,
    kt = 0.5 kn, mu = 1, lambda = 1e-3, lub_max_gap 0.5, no Brownian force."""
    return rate_params(1.0)


def _state_of(g):
    """Everything a restart needs: positions, Lees-Edwards offset, contact
    springs and the clock."""
    sc = g.scalars()
    c0, c1, dtan, _ = g.contact_states()
    return {"pos": g.particles()["pos"].copy(), "le": tuple(sc["shear_disp"]),
            "contacts": [(int(a), int(b), d) for a, b, d in zip(c0, c1, dtan)],
            "clock": (sc["time"], sc["strain"], sc["dt"], sc["shear_rate"], sc["max_velocity"],
                      sc["max_sliding_velocity"])}


def bench_cfg3(args):
    """2D monolayer: N = 8192 bidisperse discs (1:1.4, equal area shares),
    areal fraction 0.78, rate control 1r, seeded packing.  The FP32 +
    refinement form with 3 unknowns per particle (in-plane x, z translation,
    y rotation) is timed over K steps; every 100 steps (from the first) the
    run's state is handed to an FP64 engine with LF_DEM's 6x6 blocks and to
    a fresh FP32 one with 3 unknowns, both advance one step from it, and the
    largest relative velocity / stress differences are reported (the FP64
    check, outside the timed steps).  The same K steps are also timed with 6x6
    blocks in FP32 + refinement for comparison."""
    import lf_dem_gb300 as E
    from lf_dem_gb300 import build as B
    from lf_dem_gb300 import packing as PK
    n = args.count or 8192
    pk = PK.generate(n, 0.78, seed=3000, twodim=True)
    B.build()
    E.load()
    prm = monolayer_params()
    out = {}
    for label, dof in (("dof3", 3), ("dof6", 6)):
        g = E.Sim(prm, pk.position, pk.radius, pk.lx, pk.ly, pk.lz, precision=E.PREC_FP32_REFINE, dof_2d=dof)
        g.run(args.warmup)
        g.clear_step_times()
        checks = []
        ms_all = []
        run_ms = 0.0
        done = 0
        while done < args.steps:
            if dof == 3 and done % 100 == 0:
                # the FP64 check: both forms advance one step from the run's state
                st = _state_of(g)
                res = {}
                for prec, d in ((E.PREC_FP64, 6), (E.PREC_FP32_REFINE, 3)):
                    h = E.Sim(prm, st["pos"], pk.radius, pk.lx, pk.ly, pk.lz, le_disp=st["le"],
                              contacts=st["contacts"], precision=prec, dof_2d=d)
                    h.set_clock(*st["clock"])
                    h.step(calc_stress=True)
                    res[prec] = (h.particles(), h.scalars())
                    h.close()
                (p64, s64), (p32, s32) = res[E.PREC_FP64], res[E.PREC_FP32_REFINE]
                rel = lambda a, b: float(np.abs(np.asarray(a) - np.asarray(b)).max() /
                                         max(np.abs(np.asarray(b)).max(), 1e-300))
                checks.append({"step": done, "strain": float(st["clock"][1]), "vel": rel(p32["vel"], p64["vel"]),
                               "ang": rel(p32["ang"], p64["ang"]),
                               "total_stress": rel(s32["total_stress"], s64["total_stress"])})
            k = min(args.steps - done, 100 - done % 100)
            g.run(k)
            run_ms += g.timing()["run_ms"]
            ms, kern = g.step_times()
            g.clear_step_times()
            ms_all.extend(list(ms))
            done += k
        tim = g.timing()
        sc = g.scalars()
        out[label] = {"particle_steps_per_s": n * len(ms_all) / (run_ms / 1e3),
                      "ms_per_step": run_ms / len(ms_all), "p50_ms": float(np.percentile(ms_all, 50)),
                      "p99_ms": float(np.percentile(ms_all, 99)), "factor_flops": tim["factor_flops"],
                      "refine_iters": int(sc["last_refine_iters"]), "strain_reached": float(sc["strain"])}
        if checks:
            out[label]["fp64_checks"] = checks
        g.close()
    line = {"metric": "particle-steps/s, 2D monolayer N=8192 areal phi=0.78, FP32+refine (3 unknowns per particle) "
                      "with an FP64 check every 100 steps", "workload": "cfg3",
            "value": out["dof3"]["particle_steps_per_s"], "unit": "particle-steps/s", "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": out["dof3"]["ms_per_step"], "higher_is_better": True,
            "dtype": "f32+f64refine", "data": "synthetic",
            "config": {"n_particles": n, "areal_fraction": 0.78, "control": "rate 1r", "twodim": True,
                       "note": "fixed step count instead of 3 strain units; device time per step (CUDA events)"},
            **out, "speedup_dof3_vs_dof6": out["dof3"]["particle_steps_per_s"] / out["dof6"]["particle_steps_per_s"]}
    return line


def bench_serve(args):
    """Serving stream: R requests with Poisson arrivals (mean 50 ms), N
    log-uniform in [200, 16384], phi ~ U[0.45, 0.58], stress control with sigma
    log-uniform in [0.3, 100] cl, seeded packings, FP32 + refinement, each run
    to a strain target; admission by estimated factor footprint.  Reports p50
    / p99 time-to-strain (submit to done) and aggregate particle-steps/s."""
    rng = np.random.default_rng(5000)
    m = args.count or 48
    ns = np.exp(rng.uniform(np.log(200), np.log(16384), size=m)).astype(int)
    vfs = rng.uniform(0.45, 0.58, size=m)
    sig = np.exp(rng.uniform(np.log(0.3), np.log(100.0), size=m))
    arrivals = np.cumsum(rng.exponential(0.05, size=m))
    packs = gen_packings([(int(n), float(v), 5000 + k) for k, (n, v) in enumerate(zip(ns, vfs))])
    import lf_dem_gb300 as E
    from lf_dem_gb300 import build as B
    B.build()
    E.load()
    budget = int(args.hbm_budget_gb * 1e9)
    srv = E.Server(max_active=args.max_active, hbm_budget_bytes=budget)
    t0 = time.perf_counter()
    for k in range(m):
        delay = arrivals[k] - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        p = packs[k]
        srv.submit(k, stress_params(float(sig[k])), p.position, p.radius, p.lx, p.ly, p.lz,
                   strain_end=args.strain, precision=E.PREC_FP32_REFINE)
    srv.wait()
    res = srv.poll(cap=m + 8)
    st = srv.stats()
    srv.close()
    bad = [r for r in res if r.status != 0]
    tts = np.array([r.t_done - r.t_submit for r in res if r.status == 0])
    queue = np.array([r.t_admit - r.t_submit for r in res if r.status == 0])
    span = max(r.t_done for r in res) - min(r.t_submit for r in res)
    psteps = sum(r.n * r.steps for r in res if r.status == 0)
    line = {"metric": "time-to-strain p50/p99 and aggregate particle-steps/s, serving stream", "workload": "serve",
            "value": float(psteps / span), "unit": "particle-steps/s",
            "p50_time_to_strain_s": float(np.percentile(tts, 50)), "p99_time_to_strain_s": float(np.percentile(tts, 99)),
            "p50_queue_s": float(np.percentile(queue, 50)), "p99_queue_s": float(np.percentile(queue, 99)),
            "dtype": "f32+f64refine", "data": "synthetic", "failed": len(bad),
            "config": {"requests": m, "arrivals": "Poisson, mean 50 ms", "n_range": [200, 16384],
                       "phi_range": [0.45, 0.58], "sigma_cl_range": [0.3, 100], "strain_end": args.strain,
                       "max_active": args.max_active, "hbm_budget_gb": args.hbm_budget_gb,
                       "note": f"strain target {args.strain} instead of 1 strain unit"},
            "server": st, "total_steps": int(sum(r.steps for r in res)), "span_s": span}
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 form")
    ap.add_argument("--no-others", action="store_true",
                    help="skip the short cfg3 (2D monolayer), sweep and serve measurements of the default run")
    ap.add_argument("--profile", action="store_true",
                    help="profiling driver: FP32 form only, W + K steps, no measurement (for ncu)")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"], help="form used by --profile")
    ap.add_argument("--workload", default="cfg2", choices=["cfg2", "cfg3", "sweep", "serve"],
                    help="cfg2: the metric's workload (default); cfg3: the 2D monolayer; "
                         "sweep / serve: the batched and serving forms")
    ap.add_argument("--count", type=int, default=0, help="suspensions (sweep) or requests (serve)")
    ap.add_argument("--long-steps", type=int, default=1500,
                    help="steps of the run that counts pattern changes (0: skip)")
    ap.add_argument("--strain", type=float, default=0.002, help="serve: strain target of each request")
    ap.add_argument("--max-active", type=int, default=8, help="serve: concurrent requests")
    ap.add_argument("--hbm-budget-gb", type=float, default=200.0, help="serve: device bytes for admission")
    args = ap.parse_args()
    if args.workload == "cfg3":
        print(json.dumps(bench_cfg3(args)), flush=True)
        return
    if args.workload == "sweep":
        print(json.dumps(bench_sweep(args)), flush=True)
        return
    if args.workload == "serve":
        print(json.dumps(bench_serve(args)), flush=True)
        return
    if args.profile:
        import lf_dem_gb300 as E
        from lf_dem_gb300 import packing as PK
        E.load()
        pk = PK.generate(N_PART, VF, seed=2000)
        prec = E.PREC_FP32_REFINE if args.precision == "fp32" else E.PREC_FP64
        g = E.Sim(workload_params(), pk.position, pk.radius, pk.lx, pk.ly, pk.lz, precision=prec)
        g.run(args.warmup)
        g.clear_step_times()
        g.run(args.steps)
        ms, kern = g.step_times()
        t = g.timing()
        print(json.dumps({"profile_steps_ms": [float(x) for x in ms], "kernels_in_timed_steps": kern,
                          "stage_ms": t["ms"], "factor_flops": t["factor_flops"],
                          "solve_bytes": t["solve_bytes"]}))
        return
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        reference_arm(args)
        return
    world, rank, local, dist, torch = dist_setup()
    import lf_dem_gb300 as E
    from lf_dem_gb300 import build as B
    from lf_dem_gb300 import packing as PK
    if rank == 0 or world == 1:
        B.build()
    if dist is not None:
        dist.barrier()
    E.load()
    rc, name, cc, nsm = E.device_info(local)
    if rc != E.LFG_OK:
        raise SystemExit(f"no sm_103 device (rank {rank}): {name} {cc}")
    pk = PK.generate(N_PART, VF, seed=2000 + rank)
    sampler = ClockSampler(local)
    if dist is not None:
        dist.barrier()
    sampler.start()
    ms32, kern32, tim32, sc32 = run_engine(E, pk, E.PREC_FP32_REFINE, args.steps, args.warmup, local)
    clocks = sampler.stop(run_engine.window)
    # the K steps as a whole: CUDA events on the simulation's stream before the
    # first step and after the last (lfg_sim_run), host gaps between steps included
    total32 = max_over_ranks(tim32["run_ms"] / 1e3, dist, torch, f"cuda:{local}")
    value = replica_value(N_PART, args.steps, world, total32)
    res = {}
    if not args.no_fp64:
        ms64, kern64, tim64, sc64 = run_engine(E, pk, E.PREC_FP64, max(3, args.steps // 2), args.warmup, local)
        res["fp64_value"] = N_PART * tim64["run_steps"] * world / (tim64["run_ms"] / 1e3)
        res["fp64_ms_per_step"] = tim64["run_ms"] / max(tim64["run_steps"], 1)
        res["fp64_p50_ms"] = float(np.percentile(ms64, 50))
        res["fp64_p99_ms"] = float(np.percentile(ms64, 99))
        res["fp64_stage_ms"] = dict(zip(["pairs", "assembly", "factor", "solve", "forces_stress", "move"],
                                        tim64["ms"][:6]))
    if rank != 0:
        return
    hbm, bf16, bf16s, src = measured_peaks()
    # dominant kernel: the multifrontal factorisation (its launch sequence is a
    # CUDA graph); algorithmic flops per factorisation / its device time
    stage = dict(zip(["pairs", "assembly", "factor", "solve", "forces_stress", "move"], tim32["ms"][:6]))
    fact_ms = stage["factor"] / 2.0   # two factorisations per step
    achieved = tim32["factor_flops"] / (fact_ms * 1e-3) / 1e12 if fact_ms > 0 else 0.0
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            traffic = json.load(f).get("factor_fp32_bytes_per_factorisation")
    except (OSError, ValueError):
        pass
    roof = {"bound": "tensor", "achieved": achieved, "peak": bf16s, "unit": "TFLOP/s",
            "frac": achieved / bf16s, "traffic": traffic,
            "traffic_source": "profile-derived: DRAM bytes of the factorisation kernels of one factorisation, "
                              "cold caches (profiles/factorisation_and_solve_traffic_n4096_fp32.md; not measured "
                              "in this run)",
            "kernel": "FP32 multifrontal factorisation graph: k_assemble, k_scatter, k_diag, k_trsm, k_update "
                      "(CUDA cores) and k_syrk_tc (Schur complements, tcgen05 3xTF32)",
            "peak_source": f"bf16_tflops_sustained ({src}); the panel steps run on FP32 CUDA cores, "
                           "the Schur complements on the tensor cores",
            # context: FP32 CUDA-core nominal peak, 152 SMs x 128 FMA/clk x 2 x 2.07 GHz
            "fp32_simt_nominal_tflops": 80.5, "frac_of_fp32_simt_nominal": achieved / 80.5}
    solve_ms = stage["solve"]
    line = {"metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tim32["run_ms"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64refine", "data": "synthetic",
            "config": config(world), "p50_ms": float(np.percentile(ms32, 50)),
            "p99_ms": float(np.percentile(ms32, 99)), "step_events_mean_ms": float(np.mean(ms32)),
            "timing": "value and ms_per_step: one CUDA event pair around the K steps on the simulation's "
                      "stream (gaps between steps included); p50/p99 and step_events_mean_ms: an event "
                      "pair around each step",
            "stage_ms": stage, "gpu_launches": int(kern32),
            "refine_iters": sc32["last_refine_iters"], "refine_residual": sc32["last_refine_residual"],
            "symbolic_runs": sc32["n_symbolic_runs"], "roofline": roof, "clocks": clocks,
            "device": name}
    line.update(res)
    iters = max(1, int(sc32["last_refine_iters"]))
    solve_bytes_step = 2 * iters * tim32["solve_bytes"]   # predictor + corrector, one factor sweep per iteration
    line["roofline_solve"] = {"bound": "hbm", "achieved": solve_bytes_step / max(solve_ms * 1e-3, 1e-12) / 1e9,
                              "peak": hbm, "unit": "GB/s",
                              "frac": solve_bytes_step / max(solve_ms * 1e-3, 1e-12) / 1e9 / hbm,
                              "note": "factor bytes read by the triangular solves of one step / solve time"}
    line["e2e"] = run_e2e(E, pk, E.PREC_FP32_REFINE, args.steps, local)
    if args.long_steps > 0:
        line["pattern_changes"] = pattern_changes(E, pk, local, args.long_steps)
        line["pattern_changes"]["forced_rebuilds"] = rebuild_cost(E, pk, local)
    oracle_ref = None
    if not args.no_cpu:
        line["cpu_baseline"], oracle_ref = cpu_baseline(pk)
    if not args.no_fp64:
        line.update(accuracy(E, pk, local, oracle_ref))
    if not args.no_others:
        # the other configured workloads, short: the 2D monolayer (cfg3) and
        # the batched sweep (cfg4, fused and concurrent)
        import copy
        a3 = copy.copy(args)
        a3.steps, a3.warmup, a3.count = 200, 3, 0
        line["cfg3"] = bench_cfg3(a3)
        a4 = copy.copy(args)
        a4.steps, a4.warmup, a4.count, a4.sweep_modes = 5, 3, 0, ("fused", "concurrent")
        line["sweep"] = bench_sweep(a4)
        a5 = copy.copy(args)
        a5.count, a5.strain, a5.max_active, a5.hbm_budget_gb = 24, 0.0005, 8, 200.0
        line["serve"] = bench_serve(a5)
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
