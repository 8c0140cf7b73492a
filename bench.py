"""Benchmark of the GB300 angular-spectrum march.

Workload (the plain method at GPU scale, the metric's configuration):
512 x 512 x 1024 float32 grid, dX = dY = 1.5e-4 m, dT = 1e-8 s, f0 = 2 MHz,
water-like medium c0 = 1540 m/s, rho0 = 1000, beta = 3.5, alpha0 = 0.5
dB/cm/MHz (y = 1); a 20 mm piston focused at 60 mm by a quadratic delay,
5-cycle Gaussian burst, 2 MPa; Strang splitting, KT flux, frequency-weighted
and super-absorbing boundaries, dZ = 1e-4 m.  Synthetic, seeded input.

One "step" = one march step (three spectral stages over the 268 M-voxel
field, plus boundaries and accumulators).  The field (1 GiB) and its
spectrum are larger than L2, so no flush is needed between steps.

Lines printed (one JSON line):
  default         GPU arm: value = voxel-steps/s measured with CUDA events over
                  exactly K march steps after W warm-up steps; e2e through the
                  public API with host buffers; roofline of the dominant kernel;
                  CPU baseline (the oracle port on a bounded sample).
  --impl reference  the CPU reference path (the oracle port of the reference's
                  algorithm, all host threads) on a bounded sample per step.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))

NX, NY, NT = 512, 512, 1024
V = NX * NY * NT


def set_grid(nx, ny, nt):
    """Override the grid (small cases for profiler captures only)."""
    global NX, NY, NT, V
    NX, NY, NT = nx, ny, nt
    V = NX * NY * NT
B_ALG = 48.0  # algorithmic bytes per voxel-step of the Strang path (3 stages x 2 sweeps x 8 B)
# DRAM bytes (read + write) per voxel of one launch of each pass, from ncu
# captures (dram__bytes_read.sum + dram__bytes_write.sum) of the workload's
# options: the plane passes on a 512 x 512 x 256 grid (the workload's planes),
# the column passes on 256 x 256 x 1024 (its columns); the traffic scales with
# the voxel count.
DRAM_BYTES_PER_VOXEL = {"xy_A": 10.87, "xy_B": 10.90, "xy_C": 11.55, "t_nonlin": 7.25,
                        "t_mid": 7.19, "t_end": 7.22}
B_SWEEP = 8.0  # algorithmic bytes per voxel of one pass (read 4 + write 4)
METRIC = "voxel-steps/s"


def workload_params():
    from angularspectrum_heterogeneous_gb300 import SolverParams
    return SolverParams(dX=1.5e-4, dY=1.5e-4, dT=1e-8, c0=1540.0, rho0=1000.0, beta=3.5,
                        alpha0=0.5, attenPow=1.0, f0=2e6, propDist=0.07, dZmin=1e-4,
                        fluxScheme="kt", useFreqWeightedBoundary=True, useSuperAbsorbing=True)


def workload_field(grid=None):
    """Seeded synthetic input of the workload (or its central sub-grid)."""
    import scenarios as S
    nx, ny, nt = grid or (NX, NY, NT)
    return S.piston_field(nx, ny, nt, 1.5e-4, 1.5e-4, 1e-8, 2e6, 2e6, radius=20e-3,
                          focus=60e-3, ncycles=5)


def config(extra=None):
    c = {"workload": "plain KT march, 512x512x1024 focused piston 2 MPa, f0 2 MHz, "
                     "freq-weighted + super-absorbing, dZ 1e-4 m",
         "grid": [NX, NY, NT], "voxels": V, "l2": "field and spectrum (1 GiB each) exceed L2; "
                                                    "no flush needed", "parallelism": "1 GPU"}
    if extra:
        c.update(extra)
    return c


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self):
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", "0", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if r[3 + i].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# CPU baseline: the oracle port of the reference on a bounded sample
# ---------------------------------------------------------------------------
CPU_SAMPLE_GRID = (128, 128, 1024)


def cpu_march(nsteps=1, threads=None, grid=CPU_SAMPLE_GRID, max_seconds=None,
              backend="scipy"):
    """March steps of the workload's options and time axis on a central
    sub-grid of the workload (the per-voxel cost of the FFT-based march is
    nearly size independent), by the oracle port of the reference (numpy +
    scipy.fft with `threads` workers).  Operator build and one warm-up step
    excluded from the timing, as in the metric.  Returns (per-step
    voxel-steps/s list, cores, sample description)."""
    import oracle.asm_oracle as O
    threads = threads or os.cpu_count()
    if backend == "scipy":
        O.set_fft_backend("scipy", threads)
    rates = []
    try:
        p = workload_params()
        op = O.OracleParams(**{k: getattr(p, k) for k in O.OracleParams.__dataclass_fields__
                               if hasattr(p, k)})
        gx, gy, gt = grid
        u0 = workload_field(grid)  # the central crop of the workload's field
        t0 = time.time()
        m = O.OracleMarch(u0, op, "fp32").build()
        tb = time.time() - t0
        m.step()  # warm-up (allocator, FFT plans)
        t_all = time.time()
        for _ in range(nsteps):
            t0 = time.time()
            m.step()
            rates.append(gx * gy * gt / (time.time() - t0))
            if max_seconds is not None and time.time() - t_all > max_seconds:
                break
    finally:
        O.set_fft_backend("numpy")
    vox = gx * gy * gt
    return rates, threads, (
        f"march steps of the workload's options on its central {gx}x{gy}x{gt} sub-grid "
        f"({vox / 1e6:.1f} M voxels), oracle port of the reference (numpy, "
        + (f"scipy.fft workers={threads}" if backend == "scipy" else "numpy FFT, 1 thread")
        + f"), operator build ({tb:.1f} s) and one warm-up step excluded; "
        f"median of {len(rates)} step(s)")


def cpu_sample(nsteps=1, threads=None, grid=CPU_SAMPLE_GRID):
    rates, cores, sample = cpu_march(nsteps, threads, grid)
    return float(np.median(rates)), cores, sample


def run_reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    # each timed step: one march step of the CPU sample, capped at ~2 minutes
    rates, cores, sample = cpu_march(args.steps, max_seconds=120)
    v = float(np.median(rates))
    gx, gy, gt = CPU_SAMPLE_GRID
    # the same sample single-threaded (numpy's pocketfft, one core), one step
    r1, _, _ = cpu_march(1, threads=1, backend="numpy")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "voxel-steps/s",
            "n_gpus": args.gpus, "steps": len(rates), "warmup": 1,
            "ms_per_step": gx * gy * gt / v * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config({"timed_grid": list(CPU_SAMPLE_GRID)}),
            "ms_per_step_note": f"one march step of the timed {gx}x{gy}x{gt} sub-grid",
            "ms_per_step_full_grid_extrapolated": V / v * 1e3,
            "cpu_baseline": {"value": v, "unit": "voxel-steps/s", "cores": cores,
                             "kind": "port", "sample": sample},
            "cpu_single_thread": {"value": float(np.median(r1)), "unit": "voxel-steps/s",
                                  "cores": 1, "kind": "port",
                                  "sample": "one step of the same sub-grid, numpy FFT, 1 thread"},
            "e2e": {"value": v, "unit": "voxel-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# cuFFT comparison: one spectral stage through torch.fft (cuFFT)
# ---------------------------------------------------------------------------
def cufft_stage_ms(u0, reps=5):
    """One spectral stage of the march written with torch.fft (cuFFT): rfft
    along t, fft2 over (x, y), a complex multiplier, ifft2, irfft along t, on
    the workload's field resident in HBM; the median of `reps` CUDA-event
    timings after two warm-up stages.  Only a comparison: the march itself
    never calls cuFFT."""
    import torch
    u = torch.from_numpy(u0).cuda()
    nt = u.shape[2]
    g = torch.Generator(device="cuda").manual_seed(0)
    ph = torch.rand((u.shape[0], u.shape[1], nt // 2 + 1), device="cuda", generator=g)
    table = torch.polar(torch.ones_like(ph), ph * 6.283185307179586)
    del ph

    def stage(x):
        s = torch.fft.rfft(x, dim=2)
        s = torch.fft.fft2(s, dim=(0, 1))
        s *= table
        s = torch.fft.ifft2(s, dim=(0, 1))
        return torch.fft.irfft(s, n=nt, dim=2)

    for _ in range(2):
        u = stage(u)
    times = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        u = stage(u)
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    del u, table
    torch.cuda.empty_cache()
    return float(np.median(times))


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def run_gpu_arm(args):
    import torch
    from angularspectrum_heterogeneous_gb300 import Plan, angular_spectrum_solve
    from angularspectrum_heterogeneous_gb300.replicas import max_over_ranks
    from angularspectrum_heterogeneous_gb300.solver import initial_step

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    params = workload_params()
    u0 = workload_field()
    dz = initial_step(u0, params)
    plan = Plan((NX, NY, NT), params)
    plan.set_operators(0, dz)
    # launch shapes: the project's autotuner, 2 trial steps per candidate
    tuning = plan.autotune(u0, dz, steps=2) if not args.no_autotune else plan.get_tuning()
    # warm-up: W march steps
    plan.run(u0, args.warmup * dz, dz)
    # timed: exactly K march steps, CUDA events on the library's stream
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with Clocks() as clk:
        plan.run(u0, args.steps * dz, dz)
    torch.cuda.synchronize()
    ms = max_over_ranks(plan.last_run_ms(), device="cuda")
    if dist:
        dist.barrier()
    launches = sum(v[1] for v in plan.kernel_stats().values())
    # per-kernel device times (separate profiled pass of the same K steps)
    plan.set_profiling(True)
    plan.run(u0, args.steps * dz, dz)
    stats = plan.kernel_stats()
    plan.set_profiling(False)
    plan.close()
    del plan
    value = world * V * args.steps / (ms / 1e3)

    # e2e: public API, host buffers in and out, K steps; the input field in
    # page-locked host memory, two untimed calls first (host allocator warm-up;
    # the library keeps the plan of the last call with the same grid and
    # options, so the timed calls reuse it: phases_s.plan_reused).  The host
    # copies of a call vary (1 GiB each way: 5.6 ms, at times 15-60 ms), so
    # E2E_CALLS calls are timed back to back and the value is their aggregate
    # throughput (all voxel-steps over the summed wall time of every call).
    E2E_CALLS = 3
    e2e_s, h2d, d2h = float("nan"), 0, 0
    e2e_phases, e2e_calls_s = None, []
    if not args.no_e2e:
        from angularspectrum_heterogeneous_gb300.solver import host_empty
        u_host = host_empty(u0.shape, np.float32)
        u_host[...] = u0
        p2 = workload_params()
        p2.propDist = args.steps * dz
        for _ in range(2):  # host allocator warm-up: the pinned blocks return to its cache
            warm = angular_spectrum_solve(u_host, p2, verbose=False)
            del warm
        from angularspectrum_heterogeneous_gb300.solver import LAST_SOLVE_TIMINGS
        for _ in range(E2E_CALLS):
            torch.cuda.synchronize()
            t0 = time.time()
            out = angular_spectrum_solve(u_host, p2, verbose=False)
            torch.cuda.synchronize()
            e2e_calls_s.append(time.time() - t0)
            h2d = u0.nbytes / args.steps
            d2h = sum(a.nbytes for a in out) / args.steps
            e2e_phases = dict(LAST_SOLVE_TIMINGS)
            del out
        e2e_s = sum(e2e_calls_s) / E2E_CALLS
    cufft = None
    if not args.no_cufft and world == 1:
        ours = sum(stats[k][0] / stats[k][1] for k in ("xy_A", "t_mid") if stats[k][1])
        cufft = {"ms": cufft_stage_ms(u0), "ours_ms": ours,
                 "what": "one spectral stage (rfft t, fft2 xy, multiplier, ifft2, irfft t) "
                         "through torch.fft/cuFFT on the same 512x512x1024 field, against "
                         "this library's plane pass xy_A + column pass t_mid (which also "
                         "applies the taper); not part of the headline"}

    peak, peak_kind = peaks()
    kinds = {k: v for k, v in stats.items() if v[1] > 0 and k != "other"}
    dom = max(kinds, key=lambda k: kinds[k][0])
    dom_ms = kinds[dom][0] / kinds[dom][1]
    achieved = V * B_SWEEP / (dom_ms / 1e3) / 1e9
    per_kernel = {k: {"ms_per_launch": v[0] / max(v[1], 1), "launches": v[1],
                      "GBps_alg": (V * B_SWEEP / (v[0] / max(v[1], 1) / 1e3) / 1e9)
                      if v[0] > 0 else None}
                  for k, v in stats.items() if v[1] > 0}
    line = {"metric": METRIC, "value": value, "unit": "voxel-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": config({"step_ms_profiled": sum(
                v[0] for v in stats.values()) / args.steps, "tuning": tuning}),
            "hbm_GBps_alg": value * B_ALG / 1e9,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak,
                         "traffic": (DRAM_BYTES_PER_VOXEL[dom] * V
                                     if dom in DRAM_BYTES_PER_VOXEL else None),
                         "traffic_source": "ncu dram bytes per voxel (plane passes at "
                                           "512x512x256, column passes at 256x256x1024), "
                                           "scaled to the grid", "kernel": dom,
                         "peak_source": peak_kind,
                         "step_frac": value * B_ALG / 1e9 / peak},
            "kernels": per_kernel,
            "e2e": {"value": V * args.steps / e2e_s, "unit": "voxel-steps/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "calls": len(e2e_calls_s), "call_s": e2e_calls_s,
                    "phases_s": e2e_phases if not args.no_e2e else None},
            "cufft_comparison": cufft,
            "gpu_launches": int(launches),
            "clocks": clk.summary()}
    if rank == 0 and world == 1 and not args.no_cpu:
        v, cores, sample = cpu_sample(1)
        line["cpu_baseline"] = {"value": v, "unit": "voxel-steps/s", "cores": cores,
                                "kind": "port", "sample": sample}
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


# ---------------------------------------------------------------------------
# Batched workload: 64 independent focused-piston instances of uneven size
# ---------------------------------------------------------------------------
BATCH_N = 64
BATCH_CFL = 0.002  # per-column KT sub-cycling target: uneven sub-cycle counts across peaks


def batch_instances(n=BATCH_N, seed=2024):
    """Seeded instances: nX = nY in {128,192,256,384}, nT in {256,512,1024},
    focus 30-70 mm, steering +-10 deg (linear delay), peak 0.2-3 MPa; grid steps
    of the CPU-runnable case (dX = 3.08e-4 m, dT = 4e-8 s), f0 1 MHz, 15 mm
    piston, KT, Strang, Wendland taper, dZ = 2.5e-4 m."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        out.append(dict(n=int(rng.choice([128, 192, 256, 384])),
                        nt=int(rng.choice([256, 512, 1024])),
                        focus=float(rng.uniform(30e-3, 70e-3)),
                        steer=float(np.deg2rad(rng.uniform(-10.0, 10.0))),
                        p0=float(rng.uniform(0.2e6, 3e6))))
    return out


def batch_params(steps):
    from angularspectrum_heterogeneous_gb300 import SolverParams
    return SolverParams(dX=3.08e-4, dY=3.08e-4, dT=4e-8, c0=1540.0, rho0=1000.0, beta=3.5,
                        alpha0=0.5, attenPow=1.0, f0=1e6, propDist=steps * 2.5e-4,
                        dZmin=2.5e-4, fluxScheme="kt", boundaryProfile="wendland")


def batch_field(inst):
    import scenarios as S
    return S.piston_field(inst["n"], inst["n"], inst["nt"], 3.08e-4, 3.08e-4, 4e-8, 1e6,
                          inst["p0"], radius=15e-3, focus=inst["focus"], steer=inst["steer"])


def run_batch_arm(args):
    """K steps of all instances as one batched march (device time), against the
    same instances marched one plan at a time (sum of their device times)."""
    import torch
    from angularspectrum_heterogeneous_gb300.solver import Batch, _prepared_plan
    torch.cuda.set_device(0)
    insts = batch_instances()
    prm = batch_params(args.steps)
    fields = [batch_field(i) for i in insts]
    vox = sum(i["n"] * i["n"] * i["nt"] for i in insts)
    plans, dzs = [], []
    try:
        for u in fields:
            plan, dz, _ = _prepared_plan(u, prm, BATCH_CFL, 64)
            plans.append(plan)
            dzs.append(dz)
        props = [prm.propDist] * len(plans)
        # one at a time (each plan with its own step graph), after a warm-up run
        seq_ms = 0.0
        for plan, u, dz in zip(plans, fields, dzs):
            plan.run(u, args.warmup * dz, dz)
            plan.run(u, prm.propDist, dz)
            seq_ms += plan.last_run_ms()
        single = [p.outputs(("pnp", "ppp", "pI")) for p in plans]
        b = Batch(plans)
        try:
            b.run(fields, [args.warmup * d for d in dzs], dzs)  # warm-up (graph capture)
            with Clocks() as clk:
                b.run(fields, props, dzs)
            ms = b.last_run_ms()
        finally:
            b.close()
        same = all(all(np.array_equal(a, c) for a, c in zip(p.outputs(("pnp", "ppp", "pI")), s)
                       if a is not None) for p, s in zip(plans, single))
        launches = sum(sum(v[1] for v in p.kernel_stats().values()) for p in plans)
    finally:
        for p in plans:
            p.close()
    value = vox * args.steps / (ms / 1e3)
    line = {"metric": METRIC, "value": value, "unit": "voxel-steps/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": f"batched KT march of {len(insts)} focused-piston instances, "
                                   "nX=nY in {128,192,256,384}, nT in {256,512,1024}, focus "
                                   "30-70 mm, steering +-10 deg, peak 0.2-3 MPa",
                       "voxels": vox, "kt_cfl_target": BATCH_CFL, "parallelism": "1 GPU"},
            "one_at_a_time": {"value": vox * args.steps / (seq_ms / 1e3),
                              "ms_per_step": seq_ms / args.steps},
            "batch_equals_single_runs": bool(same),
            "gpu_launches": int(launches), "clocks": clk.summary()}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# Learned KT stage inside the march, on the workload's grid
# ---------------------------------------------------------------------------
LEARN_DZ, LEARN_CFL, LEARN_MIN_SUB = 5e-4, 0.01, 10
LEARN_STEPS = 120          # z = 0 .. 60 mm, through the focus of the 2 MPa piston
LEARN_PAIRS = 2 ** 21      # training column pairs (about 2e6)
NET_FLOP_PER_SAMPLE = 2 * 5 * (1 * 64 + 64 * 64 + 64 * 64 + 64 * 1)  # 83,200


def learned_params(steps):
    """The workload's medium and grid steps, KT, no boundary extras; 0.5 mm
    march steps with the KT step sub-cycled per column at CFL 0.01.  The
    reference's stability threshold guards its single KT step per march step;
    here every sub-step stays at CFL 0.01, so the threshold is lifted."""
    from angularspectrum_heterogeneous_gb300 import SolverParams
    return SolverParams(dX=1.5e-4, dY=1.5e-4, dT=1e-8, c0=1540.0, rho0=1000.0, beta=3.5,
                        alpha0=0.5, attenPow=1.0, f0=2e6, propDist=steps * LEARN_DZ,
                        dZmin=LEARN_DZ, fluxScheme="kt", stabilityThreshold=1e6)


def learned_training_pool(n_fields=8, snapshots=4, per_snapshot=65536, seed=1):
    """Columns of seeded random focused fields (peak 0.5-3 MPa, 1-3 MHz, focus
    40-80 mm, on the workload's 512x512x1024 grid) taken at `snapshots` depths
    while the plain
    GPU KT solver marches them (0.5 mm steps, per-column sub-cycling at CFL
    0.01): n_fields * snapshots * per_snapshot device columns."""
    import torch
    from angularspectrum_heterogeneous_gb300 import corrector as CR
    from angularspectrum_heterogeneous_gb300.solver import _prepared_plan, _torch_view
    rng = np.random.default_rng(seed)
    g = torch.Generator(device="cuda").manual_seed(seed)
    out = []
    for _ in range(n_fields):
        u0, f0 = CR.random_focused_field((NX, NY, NT), rng, dX=1.5e-4, dT=1e-8,
                                         focus_range=(40e-3, 80e-3))
        prm = learned_params(LEARN_STEPS)
        prm.f0 = f0
        takes = set(int(k) for k in np.linspace(LEARN_STEPS // 6, LEARN_STEPS - 1, snapshots))

        def grab(step, z, field):
            if step in takes:
                idx = torch.randint(0, NX * NY, (per_snapshot,), device="cuda", generator=g)
                out.append(field.reshape(-1, NT)[idx].clone())

        plan, dz, _ = _prepared_plan(u0, prm, LEARN_CFL, 4096)
        try:
            plan.run(u0, prm.propDist, dz,
                     lambda user, st, z, ptr: grab(st, z, _torch_view(ptr, (NX, NY, NT))))
        finally:
            plan.close()
    return torch.cat(out, 0)


def run_learned_arm(args):
    """The learned KT stage in the march of the workload's grid and 2 MPa
    piston (KT, 0.5 mm steps, z = 0..60 mm), against the plain march that
    sub-cycles every column at CFL 0.01 and the coarse march (one KT step per
    column).  The network is first trained on ~2e6 column pairs that the plain
    KT kernel generates from seeded random focused fields."""
    import torch
    from angularspectrum_heterogeneous_gb300 import corrector as CR
    from angularspectrum_heterogeneous_gb300.solver import _prepared_plan
    torch.cuda.set_device(0)
    n_coef = 3.5 / (2 * 1540.0 ** 3 * 1000.0)
    dt = 1e-8
    t0 = time.time()
    pool = learned_training_pool()
    t_pool = time.time() - t0
    net = CR.Corrector(CR.init_params(0))
    batch = 1024
    steps = LEARN_PAIRS // batch
    t0 = time.time()
    hist = CR.train(net, pool, n_coef, LEARN_DZ, dt, LEARN_CFL, steps=steps, batch=batch,
                    lr=3e-3)
    torch.cuda.synchronize()
    t_train = time.time() - t0
    del pool
    u0 = workload_field()
    prm = learned_params(LEARN_STEPS)

    def march(cfl, learned):
        plan, dz, _ = _prepared_plan(u0, prm, cfl, 4096)
        try:
            if learned:
                plan.set_learned(net, min_subcycles=LEARN_MIN_SUB, shock_ratio=0.5)
            plan.run(u0, min(args.warmup, 3) * dz, dz)  # warm-up
            with Clocks() as clk:
                plan.run(u0, prm.propDist, dz)
            ms = plan.last_run_ms()
            out = plan.outputs(("pnp", "ppp", "pI"))
            return ms, out, plan.learned_stats(), clk.summary(), plan.get_tuning()
        finally:
            plan.close()

    ms_plain, plain, _, clk, _ = march(LEARN_CFL, False)
    ms_learned, learned, (nl, ncs), _, _ = march(LEARN_CFL, True)
    from angularspectrum_heterogeneous_gb300 import ASGError
    try:  # one KT step per column: above CFL 0.5 near the focus it may not stay finite
        ms_coarse, coarse, _, _, _ = march(0.0, False)
        coarse_note = None
    except ASGError as e:
        ms_coarse, coarse, coarse_note = float("nan"), None, str(e)[:200]
    # the network alone: forward of one step's learned columns
    xr = torch.randn(max(nl // LEARN_STEPS, 1), NT, device="cuda")
    net.forward(xr)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(5):
        net.forward(xr)
    e1.record()
    torch.cuda.synchronize()
    ms_net = e0.elapsed_time(e1) / 5

    def rel(a, b):
        a = np.asarray(a, np.float64)
        b = np.asarray(b, np.float64)
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

    cx, cy = NX // 2, NY // 2
    kf = int(np.argmax(plain[2][cx, cy, :]))  # step of peak on-axis ppp
    errs = {}
    for name, out in (("learned", learned), ("coarse", coarse)):
        if out is None:
            continue
        for i, k in ((1, "pnp"), (2, "ppp"), (3, "pI")):
            errs[f"{name}_{k}"] = rel(out[i], plain[i])
            errs[f"{name}_{k}_focal_plane"] = rel(out[i][:, :, kf], plain[i][:, :, kf])
    peak_tf = None
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak_tf = float(json.load(f)["bf16_tflops"])
    except Exception:
        pass
    net_tf = xr.shape[0] * NT * NET_FLOP_PER_SAMPLE / (ms_net / 1e3) / 1e12
    vs = V * LEARN_STEPS
    line = {"metric": METRIC, "value": vs / (ms_learned / 1e3), "unit": "voxel-steps/s",
            "n_gpus": 1, "steps": LEARN_STEPS, "warmup": min(args.warmup, 3),
            "ms_per_step": ms_learned / LEARN_STEPS, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+bf16", "data": "synthetic",
            "config": {"workload": "learned KT stage in the march: 512x512x1024, 2 MPa piston "
                                   "focused at 60 mm, f0 2 MHz, KT, 0.5 mm steps over 60 mm, "
                                   "per-column sub-cycling at CFL 0.01 (plain fallback), "
                                   "learned path where >= 10 sub-cycles",
                       "train_pairs": steps * batch, "train_steps": steps,
                       "train_seconds": t_train, "pool_seconds": t_pool,
                       "final_loss": float(np.mean(hist[-20:])),
                       "learned_column_steps": int(nl), "column_steps": int(ncs)},
            "plain_kt_march": {"value": vs / (ms_plain / 1e3), "ms_per_step": ms_plain / LEARN_STEPS},
            "coarse_kt_march": ({"value": vs / (ms_coarse / 1e3),
                                 "ms_per_step": ms_coarse / LEARN_STEPS} if coarse is not None
                                else {"failed": coarse_note}),
            "speedup_vs_plain": ms_plain / ms_learned,
            "rel_l2_vs_plain_gpu_march": errs, "focal_step": kf,
            "network": {"ms": ms_net, "tflops": net_tf,
                        "frac_of_bf16_peak": (net_tf / peak_tf) if peak_tf else None,
                        "flop_per_sample": NET_FLOP_PER_SAMPLE},
            "clocks": clk}
    net.close()
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# Transcranial bowl: compact bowl source planes and synthetic skull screens
# ---------------------------------------------------------------------------
def run_hetero_arm(args):
    """Full marches (z = 0 to 80 mm) of the transcranial-bowl workload: a
    384 x 384 x 512 grid, 39 compact bowl source planes and 30 skull screens.
    One warm-up march, then 3 timed marches (CUDA events); the same march
    without screens and sources is timed beside it, and the public API call
    with host buffers gives e2e."""
    import torch
    import scenarios as S
    import angularspectrum_heterogeneous_gb300 as A
    from angularspectrum_heterogeneous_gb300.solver import _prepared_plan
    torch.cuda.set_device(0)
    t0 = time.time()
    u0, kw, screens, planes = S.tips_inputs(A, compact=True)
    t_inputs = time.time() - t0
    vox = u0.size
    reps = 3

    def params(hetero):
        p = A.SolverParams(**kw)
        if hetero:
            p.sourcePlanes, p.phaseScreens = planes, screens
        return p

    def timed(p):
        plan, dz, steps = _prepared_plan(u0, p)
        try:
            plan.run(u0, p.propDist, dz)  # warm-up march
            ms = 0.0
            with Clocks() as clk:
                for _ in range(reps):
                    plan.run(u0, p.propDist, dz)
                    ms += plan.last_run_ms()
            launches = reps * sum(v[1] for v in plan.kernel_stats().values())  # last run's
            plan.set_profiling(True)
            plan.run(u0, p.propDist, dz)
            stats = plan.kernel_stats()
        finally:
            plan.close()
        return ms / reps, len(steps), launches, stats, clk.summary()

    ms, nsteps, launches, stats, clocks = timed(params(True))
    ms_homog = timed(params(False))[0]
    # e2e: the public API with host buffers (plan, operators, screens and
    # compact sources uploaded, march, outputs read back)
    p = params(True)
    torch.cuda.synchronize()
    t0 = time.time()
    out = A.angular_spectrum_solve(u0, p, verbose=False)
    torch.cuda.synchronize()
    e2e_s = time.time() - t0
    h2d = (u0.nbytes + sum(pl.values.nbytes + pl.cols.nbytes for _, pl in planes)
           + sum(ph.nbytes + am.nbytes for _, ph, am in screens))
    d2h = sum(a.nbytes for a in out)
    peak, peak_kind = peaks()
    value = vox * nsteps / (ms / 1e3)
    kinds = {k: v for k, v in stats.items() if v[1] > 0 and k != "other"}
    line = {"metric": METRIC, "value": value, "unit": "voxel-steps/s", "n_gpus": 1,
            "steps": reps * nsteps, "warmup": nsteps, "ms_per_step": ms / nsteps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": "transcranial bowl: 384x384x512, dX 3.08e-4 m, dT 4e-8 s, "
                                   "f0 1 MHz, TIPS-like 8-element bowl (radius 46 mm, roc "
                                   "80 mm, inner 20.5 mm, focus 50 mm, 400 kPa) as compact "
                                   "source planes, synthetic skull shell screens at z 20-29 mm, "
                                   "linear water, dZ = dX, propDist 80 mm",
                       "grid": list(u0.shape), "march_steps": nsteps,
                       "source_planes": len(planes), "screens": len(screens),
                       "source_columns": int(sum(pl.cols.size for _, pl in planes)),
                       "input_build_s": t_inputs, "parallelism": "1 GPU",
                       "l2": "field and spectrum (302 MB each) exceed L2; no flush needed"},
            "homogeneous_march": {"value": vox * nsteps / (ms_homog / 1e3),
                                  "ms_per_step": ms_homog / nsteps},
            "hbm_GBps_alg": value * B_ALG / 1e9,
            "roofline": {"bound": "hbm", "step_frac": value * B_ALG / 1e9 / peak,
                         "peak": peak, "peak_source": peak_kind},
            "kernels": {k: {"ms_per_launch": v[0] / v[1], "launches": v[1]}
                        for k, v in kinds.items()},
            "e2e": {"value": vox * nsteps / e2e_s, "unit": "voxel-steps/s",
                    "h2d_bytes_per_step": h2d / nsteps, "d2h_bytes_per_step": d2h / nsteps},
            "gpu_launches": int(launches), "clocks": clocks}
    print(json.dumps(line))


def rank_launch_command(argv, n, port=None):
    """The torchrun command that runs this script as n ranks on one node (one
    per GPU, LOCAL_RANK = GPU index), rendezvous on 127.0.0.1."""
    if port is None:
        import socket
        with socket.socket() as sk:
            sk.bind(("127.0.0.1", 0))
            port = sk.getsockname()[1]
    return [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
            f"--nproc-per-node={n}", "--master-addr=127.0.0.1", f"--master-port={port}",
            os.path.abspath(__file__), *argv]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--grid", type=int, nargs=3, default=None,
                    help="profiling only: a smaller grid with the same options")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-cufft", action="store_true")
    ap.add_argument("--print-rank-env", action="store_true",
                    help="each rank prints its RANK/LOCAL_RANK/WORLD_SIZE and exits")
    ap.add_argument("--workload", default="plain",
                    choices=["plain", "batch", "learned", "hetero"],
                    help="batch: the 64-instance batched march; learned: the learned KT "
                         "step against the plain one; hetero: the transcranial bowl with "
                         "skull screens (none is the headline line)")
    args = ap.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # one process per GPU: relaunch this command under torchrun
        sys.exit(subprocess.call(rank_launch_command(sys.argv[1:], args.gpus)))
    if args.print_rank_env:
        print(json.dumps({k: os.environ.get(k) for k in
                          ("RANK", "LOCAL_RANK", "WORLD_SIZE", "MASTER_ADDR")}), flush=True)
        return
    if args.grid:
        set_grid(*args.grid)
    if args.workload == "batch" and args.impl != "reference":
        run_batch_arm(args)
        return
    if args.workload == "learned" and args.impl != "reference":
        run_learned_arm(args)
        return
    if args.workload == "hetero" and args.impl != "reference":
        run_hetero_arm(args)
        return
    if args.impl == "reference":
        run_reference_arm(args)
    else:
        run_gpu_arm(args)


if __name__ == "__main__":
    main()
