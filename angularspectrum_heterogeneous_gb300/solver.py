"""Drop-in solver API: ``SolverParams`` and ``angular_spectrum_solve``.

Same names, fields, defaults, arguments and return tuple as the reference
(``angular_spectrum_solver.py:35-76`` and ``:1217-1567``); the march itself
runs on the GPU through the C ABI of ``libasgb300.so``.

Differences from the reference, all deliberate:

* When the stability test fails (``:1420``), the reference restarts from z=0
  with a step that can never fall below ``dZmin`` and so never terminates;
  here :class:`StabilityError` is raised.
* A non-finite field raises ``ASGError(ASG_ERR_NAN)``; the reference carries
  NaNs along silently.
* ``per_step_callback`` receives a torch CUDA tensor *view* of the field
  (valid during the call; clone it to keep it) where the reference passes a
  JAX array.
* Time-of-flight extraction needs the ``tof_extraction`` module, which is not
  part of the reference tree; asking for it raises ``NotImplementedError``.
"""
from __future__ import annotations

import atexit
import ctypes as C
import dataclasses
import time as _time
from dataclasses import dataclass
from typing import Callable, Optional

import numpy as np

from . import _lib
from ._lib import ASGError, StabilityError  # noqa: F401  (re-exported)
from .operators import step_operators, step_sequence


@dataclass
class SolverParams:
    """All solver parameters (defaults as in the reference, ``:35-76``)."""
    dX: float = 0.0
    dY: float = 0.0
    dT: float = 0.0
    c0: float = 1500.0
    rho0: float = 1000.0
    beta: float = 3.5
    alpha0: float = 0.5          # dB/MHz^pow/cm  (negative -> water)
    attenPow: float = 1.0
    f0: float = 5e6
    propDist: float = 0.08
    boundaryFactor: float = 0.2
    useSplitStep: bool = True
    useAdaptiveFiltering: bool = True
    useTVD: bool = True
    freqFilterThreshold: float = 0.05
    adaptiveFilterStrength: float = 0.7
    stabilityThreshold: float = 0.2
    stabilityRecoveryFactor: float = 0.15
    dZmin: float = 1e-3
    useBoundaryLayer: bool = True
    boundaryProfile: str = 'quadratic'
    useFreqWeightedBoundary: bool = False
    useSuperAbsorbing: bool = False
    superAbsorbingStrength: float = 0.8
    fluxScheme: str = 'rusanov'
    useObliquityCorrection: bool = True
    useNonlinearityObliquity: bool = False
    phaseScreens: object = None
    sourcePlanes: object = None


def flux_kind(params) -> int:
    """Nonlinear scheme the driver dispatches to (``:1454-1492``): Lie always
    uses the standard Rusanov flux; Strang uses KT, TVD-Rusanov or Rusanov."""
    if not params.useSplitStep:
        return _lib.FLUX_RUSANOV
    if params.fluxScheme == 'kt':
        return _lib.FLUX_KT
    if params.useTVD:
        return _lib.FLUX_RUSANOV_TVD
    return _lib.FLUX_RUSANOV


def initial_step(initial_field, params) -> float:
    """dZ of the reference (``:1292-1296``): max(min(s dT / (max|u| N), dZmin), dZmin),
    or dZmin when max|u| > 0 fails (zero or NaN fields).  For every finite
    field that is dZmin, whatever max|u| is, so the field is not scanned (a
    1 GiB scan costs ~0.15 s on the host); non-finite fields are rejected by
    the run (ASG_ERR_NAN)."""
    return float(params.dZmin)


# Launch shapes chosen by Plan.autotune, per grid and option set, for this
# process: later plans with the same key start from them.
TUNING_CACHE = {}

# Host wall-clock seconds of the phases of the last angular_spectrum_solve
# call (plan and operators, march with the field upload, output read-back).
LAST_SOLVE_TIMINGS = {}

# The plan of the last angular_spectrum_solve call without phase screens or
# source planes stays alive for the next call with the same grid and
# parameters (the step sizes follow from them), which then skips the plan
# set-up and the multiplier-table build (8.5 ms at 512 x 512 x 1024).  One
# plan at a time: a call with another key closes it before building its own,
# so the device never holds two.  KEEP_LAST_PLAN = False turns this off;
# release_cached_plan() frees the plan now.
KEEP_LAST_PLAN = True
_LAST_PLAN = {"key": None, "plan": None}


def release_cached_plan():
    """Close the plan kept from the last angular_spectrum_solve call, if any."""
    plan = _LAST_PLAN["plan"]
    _LAST_PLAN.update(key=None, plan=None)
    if plan is not None:
        plan.close()


atexit.register(release_cached_plan)


def _solve_key(shape, params):
    if params.phaseScreens is not None or params.sourcePlanes is not None:
        return None
    return (tuple(shape),) + tuple(getattr(params, f.name) for f in dataclasses.fields(params)
                                   if f.name not in ("phaseScreens", "sourcePlanes"))


class Plan:
    """One GPU plan: grid, options, operators, screens and sources."""

    def __init__(self, shape, params, kt_cfl_target: float = 0.0, kt_max_subcycles: int = 1024):
        self.lib = _lib.load()
        nX, nY, nT = shape
        self.shape = (nX, nY, nT)
        self.params = params
        cfg = _lib.Config()
        cfg.nX, cfg.nY, cfg.nT = nX, nY, nT
        cfg.dX, cfg.dY, cfg.dT = params.dX, params.dY, params.dT
        cfg.c0, cfg.rho0, cfg.beta, cfg.f0 = params.c0, params.rho0, params.beta, params.f0
        cfg.split_step = int(bool(params.useSplitStep))
        cfg.flux = flux_kind(params)
        cfg.boundary_layer = int(bool(params.useBoundaryLayer))
        cfg.freq_weighted = int(bool(params.useFreqWeightedBoundary))
        cfg.super_absorbing = int(bool(params.useSuperAbsorbing))
        cfg.super_absorbing_strength = params.superAbsorbingStrength
        cfg.nonlinear_obliquity = int(bool(params.useNonlinearityObliquity))
        cfg.stability_threshold = params.stabilityThreshold
        cfg.adaptive_filter_strength = params.adaptiveFilterStrength
        cfg.kt_cfl_target = kt_cfl_target
        cfg.kt_max_subcycles = kt_max_subcycles
        cfg.pax_x, cfg.pax_y = nX // 2, nY // 2
        h = C.c_void_p()
        _lib.check(self.lib.asg_plan_create(C.byref(cfg), C.byref(h)))
        self.h = h
        self._keep = []
        self.n_screens = 0
        self.tuning_key = (self.shape, cfg.flux, cfg.split_step, cfg.freq_weighted,
                           cfg.super_absorbing, cfg.nonlinear_obliquity, kt_cfl_target > 0)
        if self.tuning_key in TUNING_CACHE:
            self.set_tuning(TUNING_CACHE[self.tuning_key])

    def get_tuning(self) -> dict:
        """Effective launch shapes (columns per block of the three column
        passes, resident-cluster cap of the plane kernel)."""
        t = _lib.Tuning()
        _lib.check(self.lib.asg_get_tuning(self.h, C.byref(t)))
        return t.as_dict()

    def set_tuning(self, tuning: dict):
        t = _lib.Tuning(**{k: int(v) for k, v in tuning.items()})
        _lib.check(self.lib.asg_set_tuning(self.h, C.byref(t)))

    def autotune(self, initial_field, dz: float, steps: int = 2) -> dict:
        """Time every launch-shape candidate on `steps` march steps from
        `initial_field`, keep the fastest and remember it for this grid and
        option set. Overwrites the plan's outputs (run afterwards)."""
        u0 = np.ascontiguousarray(initial_field, dtype=np.float32)
        assert u0.shape == self.shape
        t = _lib.Tuning()
        _lib.check(self.lib.asg_autotune(self.h, _lib.fptr(u0), float(dz), int(steps),
                                         C.byref(t)))
        TUNING_CACHE[self.tuning_key] = t.as_dict()
        return t.as_dict()

    def close(self):
        if getattr(self, "h", None):
            self.lib.asg_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_operators(self, slot: int, dz: float):
        nX, nY, nT = self.shape
        o = step_operators(self.params, nX, nY, nT, dz)
        arrs = {}

        def d(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=np.float64)
            arrs[id(a)] = a
            return _lib.dptr(a)

        s = _lib.StepOps()
        s.dz = dz
        s.kx, s.ky, s.kt = d(o.kx), d(o.ky), d(o.kt)
        s.kfilt_start, s.kfilt_max = o.kfilt_start, o.kfilt_max
        s.alpha, s.alpha_star = d(o.alpha), d(o.alpha_star)
        s.atten_obliquity = int(o.atten_obliquity)
        s.atten_clip_negative = int(o.atten_clip_negative)
        s.abl_x, s.abl_y, s.abl_t = d(o.abl_x), d(o.abl_y), d(o.abl_t)
        s.fw_exponent, s.fw_taper_x, s.fw_taper_y = d(o.fw_exponent), d(o.fw_taper_x), d(o.fw_taper_y)
        s.sa_wx, s.sa_wy = d(o.sa_wx), d(o.sa_wy)
        s.beta_tvd = o.beta_tvd
        _lib.check(self.lib.asg_set_step_operators(self.h, slot, C.byref(s)))

    def add_screen(self, z, phase, amp=None):
        ph = np.ascontiguousarray(phase, dtype=np.float32)
        am = None if amp is None else np.ascontiguousarray(amp, dtype=np.float32)
        assert ph.shape == self.shape[:2]
        _lib.check(self.lib.asg_add_screen(self.h, float(z), _lib.fptr(ph), _lib.fptr(am)))
        self.n_screens += 1

    def add_source(self, z, plane):
        """A dense (nX, nY, nT) source plane, or a ``sources.CompactPlane``."""
        from .sources import CompactPlane
        if isinstance(plane, CompactPlane):
            assert tuple(plane.shape) == self.shape
            cols = np.ascontiguousarray(plane.cols, dtype=np.int32)
            vals = np.ascontiguousarray(plane.values, dtype=np.float32)
            assert vals.shape == (cols.size, self.shape[2])
            _lib.check(self.lib.asg_add_source_compact(
                self.h, float(z), cols.ctypes.data_as(C.POINTER(C.c_int)), int(cols.size),
                _lib.fptr(vals)))
            return
        pl = np.ascontiguousarray(plane, dtype=np.float32)
        assert pl.shape == self.shape
        _lib.check(self.lib.asg_add_source(self.h, float(z), _lib.fptr(pl)))

    def run(self, initial_field, prop_dist, dz, callback=None):
        u0 = np.ascontiguousarray(initial_field, dtype=np.float32)
        assert u0.shape == self.shape
        n = C.c_int(0)
        cb = _lib.STEP_CB(callback) if callback is not None else _lib.STEP_CB()
        self._cb = cb
        _lib.check(self.lib.asg_run(self.h, _lib.fptr(u0), float(prop_dist), float(dz), cb, None,
                                    C.byref(n)))
        self.nsteps = n.value
        return self.nsteps

    def outputs(self, want=("field", "pnp", "ppp", "pI", "pIloss", "zaxis", "pax")):
        nX, nY, nT = self.shape
        nz = self.nsteps
        field = host_empty((nX, nY, nT), np.float32) if "field" in want else None
        acc = {k: (host_empty((nX, nY, nz), np.float32) if k in want else None)
               for k in ("pnp", "ppp", "pI", "pIloss")}
        zaxis = np.empty(nz, np.float64) if "zaxis" in want else None
        pax = np.empty((nT, nz), np.float32) if "pax" in want else None
        _lib.check(self.lib.asg_get_outputs(
            self.h, _lib.fptr(field), _lib.fptr(acc["pnp"]), _lib.fptr(acc["ppp"]),
            _lib.fptr(acc["pI"]), _lib.fptr(acc["pIloss"]), _lib.dptr(zaxis), _lib.fptr(pax)))
        return field, acc["pnp"], acc["ppp"], acc["pI"], acc["pIloss"], zaxis, pax

    def last_run_ms(self):
        v = C.c_double(0)
        _lib.check(self.lib.asg_last_run_ms(self.h, C.byref(v)))
        return v.value

    def set_learned(self, net, min_subcycles: int = 10, shock_ratio: float = 0.5):
        """Learned KT stage (see asg_set_learned): per column one coarse KT step
        plus the network's correction where the plain step would need at least
        `min_subcycles` sub-cycles and the column is smooth, the plain
        sub-cycled KT step elsewhere.  `net` is a corrector.Corrector (kept
        alive by the plan); None switches the stage off."""
        _lib.check(self.lib.asg_set_learned(self.h, None if net is None else net.h,
                                            int(min_subcycles), float(shock_ratio)))
        self._learned_net = net

    def learned_stats(self):
        """(columns that took the learned path, column steps) of the last run."""
        a, b = C.c_long(0), C.c_long(0)
        _lib.check(self.lib.asg_learned_stats(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def set_graphs(self, enable: bool):
        """Replay regular march steps from one captured CUDA graph (default on)."""
        _lib.check(self.lib.asg_set_graphs(self.h, int(enable)))

    def set_profiling(self, enable: bool):
        _lib.check(self.lib.asg_set_profiling(self.h, int(enable)))

    def kernel_stats(self):
        """{kind: (device ms, launches)} of the last run."""
        n = len(_lib.KERNEL_KINDS)
        ms = (C.c_double * n)()
        cnt = (C.c_long * n)()
        _lib.check(self.lib.asg_kernel_stats(self.h, ms, cnt, n))
        return {k: (ms[i], cnt[i]) for i, k in enumerate(_lib.KERNEL_KINDS)}

    def apply_operator(self, op: int, field, screen_index: int = 0):
        """One step operator on a field (see asg_apply_operator)."""
        u = np.array(field, dtype=np.float32, order="C", copy=True)
        sc = C.c_double(0.0)
        _lib.check(self.lib.asg_apply_operator(self.h, op, _lib.fptr(u), screen_index,
                                               C.byref(sc)))
        return sc.value if op == 8 else u


def host_empty(shape, dtype=np.float32):
    """An uninitialised host array in page-locked memory from torch's caching
    host allocator (a numpy view that keeps its block alive; the block goes
    back to the cache when the array is freed).  A fresh 1 GiB numpy array
    costs the OS zeroing and, for the device copy, page-locking of every
    page on each call; a cached pinned block costs neither, and the copy runs
    at the host link's full rate.  Plain numpy memory if no device is there."""
    global HOST_EMPTY_FALLBACKS
    try:
        import torch
        if torch.cuda.is_available():
            td = {np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64}
            return torch.empty(tuple(shape), dtype=td[np.dtype(dtype)], pin_memory=True).numpy()
    except (ImportError, KeyError, RuntimeError) as e:
        HOST_EMPTY_FALLBACKS += 1
        LAST_SOLVE_TIMINGS["host_alloc_fallback"] = str(e)[:200]
    return np.empty(shape, dtype)


# allocations host_empty could not page-lock (plain numpy memory instead)
HOST_EMPTY_FALLBACKS = 0


def _torch_view(ptr, shape):
    import torch

    class _Dev:
        __cuda_array_interface__ = {
            "shape": tuple(shape), "typestr": "<f4", "data": (int(ptr), False), "version": 3,
        }
    return torch.as_tensor(_Dev(), device="cuda")


def _prepared_plan(u0, params, kt_cfl_target=0.0, kt_max_subcycles=1024):
    """A plan with the step operators (regular and partial step), screens and
    sources of one solve; returns (plan, dZ, step sequence)."""
    dz = initial_step(u0, params)
    steps = step_sequence(params.propDist, dz)
    plan = Plan(u0.shape, params, kt_cfl_target=kt_cfl_target, kt_max_subcycles=kt_max_subcycles)
    try:
        plan.set_operators(0, dz)
        partial = [s for s in steps if abs(s - dz) > 1e-15]
        if partial:
            plan.set_operators(1, partial[-1])
        if params.phaseScreens is not None:
            for scr in params.phaseScreens:
                amp = scr[2] if len(scr) > 2 else None
                plan.add_screen(scr[0], scr[1], amp)
        if params.sourcePlanes is not None:
            for z, plane in params.sourcePlanes:
                plan.add_source(z, plane)
    except Exception:
        plan.close()
        raise
    return plan, dz, steps


class Batch:
    """Independent plans (grids of any size) marched together: every batch
    step of the plans' regular steps is one CUDA-graph launch that forks to
    all plans' streams (see asg_batch_run)."""

    def __init__(self, plans):
        self.lib = _lib.load()
        self.plans = list(plans)
        arr = (C.c_void_p * len(self.plans))(*[p.h.value for p in self.plans])
        h = C.c_void_p()
        _lib.check(self.lib.asg_batch_create(arr, len(self.plans), C.byref(h)))
        self.h = h

    def set_learned(self, net, min_subcycles: int = 10, shock_ratio: float = 0.5):
        """Learned KT stage (see asg_set_learned): per column one coarse KT step
        plus the network's correction where the plain step would need at least
        `min_subcycles` sub-cycles and the column is smooth, the plain
        sub-cycled KT step elsewhere.  `net` is a corrector.Corrector (kept
        alive by the plan); None switches the stage off."""
        _lib.check(self.lib.asg_set_learned(self.h, None if net is None else net.h,
                                            int(min_subcycles), float(shock_ratio)))
        self._learned_net = net

    def learned_stats(self):
        """(columns that took the learned path, column steps) of the last run."""
        a, b = C.c_long(0), C.c_long(0)
        _lib.check(self.lib.asg_learned_stats(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def set_graphs(self, enable: bool):
        _lib.check(self.lib.asg_batch_set_graphs(self.h, int(enable)))

    def run(self, fields, prop_dists, dzs):
        n = len(self.plans)
        us = [np.ascontiguousarray(f, dtype=np.float32) for f in fields]
        for u, p in zip(us, self.plans):
            assert u.shape == p.shape
        fp = (C.POINTER(C.c_float) * n)(*[_lib.fptr(u) for u in us])
        pd = (C.c_double * n)(*[float(x) for x in prop_dists])
        dd = (C.c_double * n)(*[float(x) for x in dzs])
        ns = (C.c_int * n)()
        _lib.check(self.lib.asg_batch_run(self.h, fp, pd, dd, ns))
        for p, k in zip(self.plans, ns):
            p.nsteps = k
        return list(ns)

    def last_run_ms(self):
        v = C.c_double(0)
        _lib.check(self.lib.asg_batch_last_run_ms(self.h, C.byref(v)))
        return v.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.asg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def solve_batch(initial_fields, params_list, kt_cfl_target: float = 0.0,
                kt_max_subcycles: int = 1024, return_timing: bool = False):
    """`angular_spectrum_solve` of many independent instances (uneven grids
    allowed) in one batched march.  Returns one output tuple per instance,
    each exactly as `angular_spectrum_solve` returns it (and the device time
    of the march in ms with return_timing)."""
    if len(initial_fields) != len(params_list):
        raise ValueError("one parameter set per initial field")
    plans, dzs, us = [], [], []
    try:
        for f, prm in zip(initial_fields, params_list):
            u0 = np.ascontiguousarray(f, dtype=np.float32)
            if u0.ndim != 3:
                raise ValueError("initial_field must be (nX, nY, nT)")
            plan, dz, _ = _prepared_plan(u0, prm, kt_cfl_target, kt_max_subcycles)
            plans.append(plan)
            dzs.append(dz)
            us.append(u0)
        batch = Batch(plans)
        try:
            batch.run(us, [prm.propDist for prm in params_list], dzs)
            outs = [p.outputs() for p in plans]
            ms = batch.last_run_ms()
        finally:
            batch.close()
        return (outs, ms) if return_timing else outs
    finally:
        for p in plans:
            p.close()


def angular_spectrum_solve(
        initial_field: np.ndarray,
        params: SolverParams,
        verbose: bool = True,
        per_step_callback: Optional[Callable] = None,
        tof_ref_trace: Optional[np.ndarray] = None,
        tof_t_ref_peak_s: Optional[float] = None,
        tof_env_ratio: Optional[float] = None,
        taxis: Optional[np.ndarray] = None):
    """Propagate a 3-D field with the modified angular spectrum method on the GPU.

    Returns ``(field, pnp, ppp, pI, pIloss, zaxis, pax)`` exactly as the
    reference does (``:1556-1567``): field (nX,nY,nT) float32, pnp/ppp/pI/pIloss
    (nX,nY,nZ) float32, zaxis (nZ,) float64, pax (nT,nZ) float32.
    """
    if tof_ref_trace is not None and tof_t_ref_peak_s is None:
        raise ValueError('tof_t_ref_peak_s is required when tof_ref_trace is provided')
    if tof_ref_trace is not None or tof_env_ratio is not None:
        raise NotImplementedError(
            "time-of-flight extraction needs the tof_extraction module, which is not part of "
            "the reference tree")
    u0 = np.ascontiguousarray(initial_field, dtype=np.float32)
    if u0.ndim != 3:
        raise ValueError("initial_field must be (nX, nY, nT)")
    nX, nY, nT = u0.shape
    t_start = _time.perf_counter()
    LAST_SOLVE_TIMINGS.clear()
    key = _solve_key(u0.shape, params) if KEEP_LAST_PLAN else None
    reused = key is not None and _LAST_PLAN["key"] == key
    if reused:
        plan = _LAST_PLAN["plan"]
        _LAST_PLAN.update(key=None, plan=None)
        dz = initial_step(u0, params)
        steps = step_sequence(params.propDist, dz)
    else:
        release_cached_plan()
        plan, dz, steps = _prepared_plan(u0, params)
    keep = False
    try:
        cb = None
        if per_step_callback is not None:
            def cb(user, step, z, ptr):
                per_step_callback(step, z, _torch_view(ptr, (nX, nY, nT)))
        t0 = _time.time()
        t_plan = _time.perf_counter()
        plan.run(u0, params.propDist, dz, cb)
        t_run = _time.perf_counter()
        out = plan.outputs()
        t_out = _time.perf_counter()
        LAST_SOLVE_TIMINGS.update(plan_s=t_plan - t_start, run_s=t_run - t_plan,
                                  march_device_s=plan.last_run_ms() / 1e3,
                                  outputs_s=t_out - t_run,
                                  host_alloc_fallbacks=HOST_EMPTY_FALLBACKS,
                                  plan_reused=reused)
        if verbose:
            z = 0.0
            for cc, d in enumerate(steps):
                print(f'z = {z + d:.6f} m  (step {cc})')
                z += d
            print(f'Simulation completed in {_time.time() - t0:.2f} s  ({len(steps)} steps)')
        keep = key is not None
        return out
    finally:
        if keep:
            _LAST_PLAN.update(key=key, plan=plan)
        else:
            plan.close()
