"""Generate the golden fixtures from the reference implementation itself.

The reference (`angular_spectrum_solver.py`, a JAX module) cannot be imported
as shipped in a machine without JAX: it imports ``jax`` and a missing
``tof_extraction`` module.  This script installs a small numpy-backed stand-in
for the handful of ``jax``/``jax.numpy`` names the module uses
(``jit`` -> identity, ``jnp.*`` -> numpy, functional ``.at[idx].set/add``
updates) and a stub ``tof_extraction``, imports the reference from the
directory given by ``--reference-dir`` or the ``ASG_REFERENCE_DIR``
environment variable (one of them is required), runs a fixed set of seeded
small scenarios and writes the inputs and outputs to ``*.npz`` files next to
this script.

The fixtures are small on purpose (a few hundred KB in total) and are
committed; the GPU tests never need the reference.  Two precisions are
produced: ``fp32`` runs the module as shipped; ``fp64`` remaps the module's
float32/complex64 casts to float64/complex128 (the FP64 oracle).

Run:  python tests/golden/make_golden.py  --reference-dir DIR
      (or ASG_REFERENCE_DIR=DIR python tests/golden/make_golden.py)
"""
from __future__ import annotations

import argparse
import importlib
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


# ---------------------------------------------------------------------------
# numpy stand-in for the jax names the reference uses
# ---------------------------------------------------------------------------
class _AtIndexer:
    def __init__(self, arr):
        self._arr = arr

    def __getitem__(self, idx):
        return _AtUpdate(self._arr, idx)


class _AtUpdate:
    def __init__(self, arr, idx):
        self._arr, self._idx = arr, idx

    def set(self, value):
        out = np.array(self._arr, copy=True).view(JArray)
        out[self._idx] = value
        return out

    def add(self, value):
        base = np.asarray(self._arr)
        upd = base[self._idx] + np.asarray(value)
        dt = np.result_type(base.dtype, np.asarray(upd).dtype)
        out = np.array(base, dtype=dt, copy=True).view(JArray)
        out[self._idx] = upd
        return out


class JArray(np.ndarray):
    """ndarray with the functional ``.at[...]`` update syntax of jax arrays."""

    @property
    def at(self):
        return _AtIndexer(self)


def _wrap(x):
    if isinstance(x, np.ndarray) and not isinstance(x, JArray):
        return x.view(JArray)
    return x


def _make_jax_modules(fp64: bool):
    def remap(dt):
        if not fp64 or dt is None:
            return dt
        dt = np.dtype(dt)
        if dt == np.float32:
            return np.float64
        if dt == np.complex64:
            return np.complex128
        return dt

    jnp = types.ModuleType("jax.numpy")
    passthrough = [
        "abs", "maximum", "minimum", "sign", "exp", "power", "clip", "real",
        "sum", "zeros_like", "ceil", "max", "where", "pad", "sqrt", "arange",
        "newaxis", "pi", "mean", "ones_like", "conj", "imag", "min",
    ]
    for name in passthrough:
        obj = getattr(np, name)
        if callable(obj):
            def _f(*a, _o=obj, **k):
                if "dtype" in k:
                    k["dtype"] = remap(k["dtype"])
                return _wrap(_o(*a, **k))
            setattr(jnp, name, _f)
        else:
            setattr(jnp, name, obj)
    jnp.float32 = np.float64 if fp64 else np.float32
    jnp.complex64 = np.complex128 if fp64 else np.complex64
    jnp.float64 = np.float64
    jnp.complex128 = np.complex128
    jnp.ndarray = np.ndarray

    def array(x, dtype=None):
        return _wrap(np.array(x, dtype=remap(dtype), copy=True))
    jnp.array = array

    fft = types.ModuleType("jax.numpy.fft")
    for name in ["fft", "ifft", "rfft", "irfft", "fft2", "ifft2", "fftn", "ifftn",
                 "fftshift", "ifftshift", "rfftfreq", "fftfreq"]:
        def _g(*a, _o=getattr(np.fft, name), **k):
            return _wrap(_o(*a, **k))
        setattr(fft, name, _g)
    jnp.fft = fft

    jax = types.ModuleType("jax")
    jax.numpy = jnp

    def jit(f=None, **kw):
        if f is None:
            return lambda g: g
        return f
    jax.jit = jit
    jax.config = types.SimpleNamespace(update=lambda *a, **k: None)
    return jax, jnp, fft


def load_reference(reference_dir: str, fp64: bool):
    for m in ["angular_spectrum_solver", "jax", "jax.numpy", "jax.numpy.fft", "tof_extraction"]:
        sys.modules.pop(m, None)
    jax, jnp, fft = _make_jax_modules(fp64)
    sys.modules["jax"] = jax
    sys.modules["jax.numpy"] = jnp
    sys.modules["jax.numpy.fft"] = fft
    tof = types.ModuleType("tof_extraction")
    tof.extract_tof_envelope = lambda *a, **k: None
    tof.extract_tof_matched_filter_parabolic = lambda *a, **k: None
    sys.modules["tof_extraction"] = tof
    if reference_dir not in sys.path:
        sys.path.insert(0, reference_dir)
    mod = importlib.import_module("angular_spectrum_solver")
    return mod


# ---------------------------------------------------------------------------
# Scenario inputs (seeded; shared with the tests through scenarios.py)
# ---------------------------------------------------------------------------
sys.path.insert(0, HERE)
import scenarios as S  # noqa: E402


def _np(x):
    return np.asarray(x)


def gen_operators(ref, out):
    """Operator builders at small odd/even shapes."""
    for (nX, nY, nT) in [(8, 10, 12), (7, 9, 11)]:
        tag = f"{nX}x{nY}x{nT}"
        dX, dY, dT, c0 = 2.0e-4, 2.5e-4, 3.0e-8, 1540.0
        for ss in (False, True):
            for af in (False, True):
                HH, HHh = ref.precalculate_mas(nX, nY, nT, dX, dY, 1.0e-4, dT, c0,
                                               split_step=ss, adaptive_filtering=af,
                                               filter_threshold=0.05, filter_strength=0.7)
                out[f"mas_{tag}_ss{int(ss)}_af{int(af)}_HH"] = HH
                if ss:
                    out[f"mas_{tag}_ss{int(ss)}_af{int(af)}_HHhalf"] = HHh
        for prof in ("quadratic", "wendland"):
            abl, ablh = ref.precalculate_abl(nX, nY, nT, 0.2, split_step=True, profile=prof)
            out[f"abl_{tag}_{prof}"] = abl
            out[f"ablhalf_{tag}_{prof}"] = ablh
            out[f"ablfreq_{tag}_{prof}"] = ref.precalculate_abl_freq(
                nX, nY, nT, dT, c0, 1.0e6, boundary_factor=0.2, profile=prof)
        for obl in (False, True):
            a, ah = ref.precalculate_ad(2.17e-3, nX, nY, nT, dX, dY, 1.0e-4, dT, c0, 1e6,
                                        split_step=True, obliquity=obl)
            out[f"adwater_{tag}_obl{int(obl)}"] = a
            out[f"adwater_{tag}_obl{int(obl)}_half"] = ah
            for pw in (1.0, 2.0, 1.5):
                a, ah, f, alpha, disp = ref.precalculate_ad_pow2(
                    0.5, nX, nY, nT, dX, dY, 1.0e-4, dT, c0, 1e6, pw,
                    split_step=True, obliquity=obl)
                out[f"adpow_{tag}_pw{pw}_obl{int(obl)}"] = a
                out[f"adpow_{tag}_pw{pw}_obl{int(obl)}_half"] = ah
                out[f"adpow_{tag}_pw{pw}_disp"] = disp
        out[f"oblmap_{tag}"] = ref.precalculate_obliquity_map(nX, nY, nT, dX, dY, dT, c0)
        out[f"bdyw_{nX}_2"] = ref._make_boundary_weights(nX, 2)
    for n, bw in [(16, 3), (17, 4), (5, 1)]:
        out[f"ablvec_{n}_{bw}"] = ref.ablvec(n, bw)
        out[f"ablvecw_{n}_{bw}"] = ref.ablvec_wendland(n, bw)


def gen_steps(ref, out, fp64):
    """Each step kernel on a seeded small field."""
    dt = np.float64 if fp64 else np.float32
    ct = np.complex128 if fp64 else np.complex64
    for shape in [(8, 10, 16), (7, 9, 15)]:
        nX, nY, nT = shape
        tag = f"{nX}x{nY}x{nT}"
        u = S.seeded_field(shape, seed=1, amp=2.0e6).astype(dt)
        out[f"in_{tag}"] = u
        dX, dY, dT, c0, dZ = 2.0e-4, 2.5e-4, 3.0e-8, 1540.0, 1.0e-4
        HH, HHh = ref.precalculate_mas(nX, nY, nT, dX, dY, dZ, dT, c0, split_step=True,
                                       adaptive_filtering=True)
        abl, ablh = ref.precalculate_abl(nX, nY, nT, 0.2, split_step=True, profile="wendland")
        out[f"diff_{tag}"] = _np(ref._angular_spectrum_step(
            ref.jnp.array(u), ref.jnp.array(HHh, dtype=ct), ref.jnp.array(ablh, dtype=dt)))
        a, ah, _, _, _ = ref.precalculate_ad_pow2(0.5, nX, nY, nT, dX, dY, dZ, dT, c0, 1e6, 1.0,
                                                   split_step=True)
        nf = nT // 2 + 1
        out[f"atten_{tag}"] = _np(ref._attenuation_step(
            ref.jnp.array(u), ref.jnp.array(ah[:, :, :nf], dtype=ct)))
        af = ref.precalculate_abl_freq(nX, nY, nT, dT, c0, 1e6, 0.2, "wendland")
        out[f"freqw_{tag}"] = _np(ref._freq_weighted_boundary_step(
            ref.jnp.array(u), ref.jnp.array(af, dtype=dt)))
        wx = ref._make_boundary_weights(nX, max(round(nX * 0.2), 1))
        wy = ref._make_boundary_weights(nY, max(round(nY * 0.2), 1))
        out[f"superabs_{tag}"] = _np(ref._super_absorbing_step(
            ref.jnp.array(u), ref.jnp.array(wx, dtype=dt), ref.jnp.array(wy, dtype=dt),
            dX, dY, dT, c0, 0.8))
        rng = np.random.default_rng(7)
        ph = (rng.standard_normal((nX, nY)) * 1.5).astype(np.float32)
        amp = rng.uniform(0.3, 1.2, (nX, nY)).astype(np.float32)
        out[f"screen_phase_{tag}"] = ph
        out[f"screen_amp_{tag}"] = amp
        f0_bin = 1e6 / (1.0 / (nT * dT))
        out[f"screen_{tag}"] = _np(ref._apply_phase_screen(
            ref.jnp.array(u), ref.jnp.array(ph, dtype=dt), f0_bin, ref.jnp.array(amp, dtype=dt)))
        out[f"screen_noamp_{tag}"] = _np(ref._apply_phase_screen(
            ref.jnp.array(u), ref.jnp.array(ph, dtype=dt), f0_bin, None))
        obl = ref.precalculate_obliquity_map(nX, nY, nT, dX, dY, dT, c0)
        out[f"oblscalar_{tag}"] = np.asarray(float(ref._beam_obliquity_scalar(
            ref.jnp.array(u), ref.jnp.array(obl, dtype=dt))))
    # flux kernels on single columns, including a shocked profile and ragged lengths
    N = 3.5 / (2 * 1540.0 ** 3 * 1000.0)
    for nT in (64, 65, 3, 801):
        col = S.seeded_column(nT, seed=nT).astype(dt)
        out[f"col_{nT}"] = col
        f = ref.jnp.array(col.reshape(1, 1, nT))
        for dZ, dTt in [(1.0e-4, 1.0e-8), (5.0e-4, 2.0e-8)]:
            t = f"{nT}_{dZ:g}_{dTt:g}"
            out[f"rus_{t}"] = _np(ref._rusanov_flux_standard(f, N, dZ, dTt))
            out[f"tvd_{t}"] = _np(ref._rusanov_flux_tvd(f, N, dZ, dTt, 1.7))
            out[f"kt_{t}"] = _np(ref._kt_flux(f, N, dZ, dTt))
            out[f"ktmm_{t}"] = _np(ref._kt_flux_minmod(f, N, dZ, dTt))
            out[f"ktad_{t}"] = _np(ref._kt_flux_adaptive(f, N, dZ, dTt, cfl_target=0.05))


def gen_solves(ref, out, fp64, which=None):
    for name, sc in S.SOLVE_SCENARIOS.items():
        if which is not None and name not in which:
            continue
        u0, kw, extras = S.build_solve_inputs(name, ref_module=ref)
        params = ref.SolverParams(**kw)
        for k, v in extras.items():
            setattr(params, k, v)
        res = ref.angular_spectrum_solve(u0, params, verbose=False)
        keys = ["field", "pnp", "ppp", "pI", "pIloss", "zaxis", "pax"]
        for k, v in zip(keys, res):
            out[f"solve_{name}_{k}"] = np.asarray(v)


def gen_builders(ref, out):
    x = (np.arange(24) - 11.5) * 1.0e-3
    y = (np.arange(20) - 9.5) * 1.2e-3
    t = (np.arange(32) - 16) * 8e-8
    planes, depth = ref.make_bowl_source_planes(x, y, t, 1e6, 1540.0, 4e5, 10e-3, 25e-3,
                                                1.0e-3, inner_radius=3e-3, focus=20e-3,
                                                n_elements=3)
    out["bowl_planes_z"] = np.array([p[0] for p in planes])
    out["bowl_planes_f"] = np.stack([p[1] for p in planes])
    out["bowl_depth"] = np.asarray(depth)
    out["bowl_single"] = ref.make_bowl_source(x, y, t, 1e6, 1540.0, 4e5, 10e-3, 25e-3,
                                              inner_radius=3e-3, focus=20e-3, n_elements=3,
                                              element_delays=[0.0, 1e-7, 2e-7])
    ps, cm = ref.generate_phase_screen(16, 12, 1e-3, 1.2e-3, 1540.0, 1e6, 3e-3, 40.0,
                                       thickness=2e-3, seed=11)
    out["gps_phase"] = ps
    out["gps_cmap"] = cm


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference-dir", default=os.environ.get("ASG_REFERENCE_DIR"),
                    help="directory holding angular_spectrum_solver.py (or ASG_REFERENCE_DIR)")
    ap.add_argument("--only", default=None, help="comma list of solve scenarios")
    args = ap.parse_args()
    if not args.reference_dir:
        ap.error("give --reference-dir or set ASG_REFERENCE_DIR")
    which = args.only.split(",") if args.only else None
    for fp64 in (False, True):
        ref = load_reference(args.reference_dir, fp64)
        ref.jnp = sys.modules["jax.numpy"]
        out = {}
        import contextlib
        import io
        with contextlib.redirect_stdout(io.StringIO()):
            if not fp64:
                gen_operators(ref, out)
                gen_builders(ref, out)
            gen_steps(ref, out, fp64)
            gen_solves(ref, out, fp64, which)
        tag = "fp64" if fp64 else "fp32"
        path = os.path.join(HERE, f"golden_{tag}.npz")
        np.savez_compressed(path, **out)
        print(f"wrote {path}: {len(out)} arrays, {os.path.getsize(path) / 1024:.0f} KB")


if __name__ == "__main__":
    main()
