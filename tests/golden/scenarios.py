"""Seeded small scenarios shared by the golden-fixture generator and the tests.

Everything here is plain numpy.  The solve scenarios cover every option
branch of the reference driver (``angular_spectrum_solver.py:1413-1550``):
Strang/Lie splitting, Rusanov standard/TVD and KT fluxes, quadratic and
Wendland tapers, no boundary layer, water and power-law attenuation
(odd, even and fractional exponent), obliquity on/off, adaptive k-filter
on/off, frequency-weighted and super-absorbing boundaries, phase screens
(2- and 3-tuples), dense source planes (one exactly on a step boundary),
beam-obliquity nonlinearity, odd grid sizes and a partial last step.
"""
from __future__ import annotations

import numpy as np

C0 = 1540.0
RHO0 = 1000.0


def seeded_field(shape, seed, amp):
    """Smooth random band-limited field (X, Y, T) with a pulse-like time profile."""
    rng = np.random.default_rng(seed)
    nX, nY, nT = shape
    t = np.arange(nT) - (nT - 1) / 2.0
    env = np.exp(-(t / (0.22 * nT)) ** 4)
    base = rng.standard_normal(shape) * 0.3
    # cheap smoothing along t keeps the fluxes in their smooth regime mostly
    k = np.array([0.25, 0.5, 0.25])
    for _ in range(2):
        base = k[0] * np.roll(base, 1, axis=2) + k[1] * base + k[2] * np.roll(base, -1, axis=2)
    carrier = np.sin(2 * np.pi * t / 6.0)
    u = amp * (base + carrier[None, None, :]) * env[None, None, :]
    return u


def seeded_column(nT, seed):
    """A 1-D column with a smooth part, a jump (shock) and a flat stretch."""
    rng = np.random.default_rng(seed)
    t = np.linspace(-1.0, 1.0, nT)
    u = 6.0e6 * np.sin(4 * np.pi * t) * np.exp(-(2 * t) ** 4)
    if nT >= 8:
        j = nT // 3
        u[j:j + max(1, nT // 10)] += 4.0e6
        u[-max(1, nT // 8):] = 0.0
    u += rng.standard_normal(nT) * 1.0e4
    return u


def piston_field(nX, nY, nT, dX, dY, dT, f0, p0, radius, focus, ncycles=3, dur=2,
                 c0=C0, steer=0.0):
    """Circular piston focused by a quadratic delay r^2/(2 F c0), Gaussian burst.

    The temporal envelope follows the reference's initial-condition helper
    (``validate_solver.py:41-57``): exp(-(1.05 t w0/(ncycles pi))^(2 dur)) sin(w0 t).
    ``steer`` adds a linear delay x*sin(steer)/c0 (radians).
    """
    x = (np.arange(nX) - (nX - 1) / 2.0) * dX
    y = (np.arange(nY) - (nY - 1) / 2.0) * dY
    t = np.arange(nT) * dT
    t = t - t.mean()
    X, Y = np.meshgrid(x, y, indexing="ij")
    r2 = X ** 2 + Y ** 2
    ap = r2 <= radius ** 2
    # converging wave: the rim fires first (pulse centre at t = -delay)
    delay = (r2 / (2.0 * focus * c0)) + X * np.sin(steer) / c0
    delay = np.where(ap, delay - delay[ap].mean() if ap.any() else 0.0, 0.0)
    w0 = 2 * np.pi * f0
    out = np.zeros((nX, nY, nT), np.float32)
    ix, iy = np.nonzero(ap)
    for s0 in range(0, ix.size, 4096):  # aperture pixels only, in chunks
        sl = slice(s0, s0 + 4096)
        tt = t[None, :] + delay[ix[sl], iy[sl]][:, None]
        env = np.exp(-(1.05 * tt * w0 / (ncycles * np.pi)) ** (2 * dur))
        out[ix[sl], iy[sl], :] = (env * np.sin(w0 * tt) * p0).astype(np.float32)
    return out


def _screens(nX, nY, seed, zs, with_amp):
    rng = np.random.default_rng(seed)
    out = []
    for z, a in zip(zs, with_amp):
        ph = (rng.standard_normal((nX, nY)) * 0.8).astype(np.float32)
        if a:
            amp = rng.uniform(0.5, 1.1, (nX, nY)).astype(np.float32)
            out.append((z, ph, amp))
        else:
            out.append((z, ph))
    return out


def _sources(nX, nY, nT, dT, f0, zs, seed):
    rng = np.random.default_rng(seed)
    out = []
    t = np.arange(nT) * dT
    t = t - t.mean()
    w0 = 2 * np.pi * f0
    for i, z in enumerate(zs):
        m = (rng.uniform(size=(nX, nY)) < 0.15)
        d = rng.uniform(-2e-7, 2e-7, (nX, nY))
        env = np.exp(-(1.05 * (t[None, None, :] - d[:, :, None]) * w0 / (3 * np.pi)) ** 4)
        f = m[:, :, None] * env * np.sin(w0 * (t[None, None, :] - d[:, :, None])) * 3e5
        out.append((z, f.astype(np.float32)))
    return out


BASE = dict(dX=2.5e-4, dY=2.5e-4, dT=4.0e-8, c0=C0, rho0=RHO0, beta=3.5, alpha0=0.5,
            attenPow=1.0, f0=2.0e6, dZmin=2.5e-4, propDist=2.0e-3)

SOLVE_SCENARIOS = {
    # configs[0] option set, downscaled: Strang + TVD Rusanov + Wendland
    "strang_tvd_wendland": dict(shape=(16, 16, 48), p0=4e6,
                                kw=dict(fluxScheme="rusanov", boundaryProfile="wendland")),
    # configs[1] option set: KT + freq-weighted + super-absorbing
    "strang_kt_fw_sa": dict(shape=(16, 14, 64), p0=8e6,
                            kw=dict(fluxScheme="kt", useFreqWeightedBoundary=True,
                                    useSuperAbsorbing=True, f0=2.0e6)),
    "lie_water_quadratic": dict(shape=(16, 16, 40), p0=3e6,
                                kw=dict(useSplitStep=False, alpha0=-1.0)),
    "strang_std_nofilter": dict(shape=(14, 16, 48), p0=3e6,
                                kw=dict(useTVD=False, useAdaptiveFiltering=False,
                                        useObliquityCorrection=False)),
    "screens_sources": dict(shape=(16, 16, 48), p0=2e6,
                            kw=dict(fluxScheme="rusanov", boundaryProfile="wendland"),
                            screens=dict(zs=[3.0e-4, 7.5e-4, 1.1e-3], amp=[False, True, True]),
                            sources=dict(zs=[1.0e-4, 5.0e-4, 1.6e-3])),
    "kt_obliquity_nl": dict(shape=(16, 16, 48), p0=6e6,
                            kw=dict(fluxScheme="kt", useNonlinearityObliquity=True)),
    "odd_partial": dict(shape=(15, 13, 45), p0=5e6,
                        kw=dict(fluxScheme="kt", propDist=1.8e-3, dX=2.7e-4, dY=2.3e-4)),
    "noabl_pow2": dict(shape=(16, 12, 32), p0=2e6,
                       kw=dict(useBoundaryLayer=False, attenPow=2.0, alpha0=0.3)),
    "pow15_sa_only": dict(shape=(12, 16, 36), p0=3e6,
                          kw=dict(attenPow=1.5, alpha0=0.7, useSuperAbsorbing=True,
                                  superAbsorbingStrength=0.5, useTVD=False)),
    "lie_fw_kt_ignored": dict(shape=(16, 16, 33), p0=4e6,
                              kw=dict(useSplitStep=False, fluxScheme="kt",
                                      useFreqWeightedBoundary=True,
                                      boundaryProfile="wendland")),
}


def build_solve_inputs(name, ref_module=None):
    """Return (initial_field float32, SolverParams kwargs, extras) for a scenario."""
    sc = SOLVE_SCENARIOS[name]
    kw = dict(BASE)
    kw.update(sc["kw"])
    nX, nY, nT = sc["shape"]
    u0 = piston_field(nX, nY, nT, kw["dX"], kw["dY"], kw["dT"], kw["f0"], sc["p0"],
                      radius=0.35 * min(nX * kw["dX"], nY * kw["dY"]), focus=6e-3)
    extras = {}
    if "screens" in sc:
        extras["phaseScreens"] = _screens(nX, nY, 5, sc["screens"]["zs"], sc["screens"]["amp"])
    if "sources" in sc:
        extras["sourcePlanes"] = _sources(nX, nY, nT, kw["dT"], kw["f0"],
                                          sc["sources"]["zs"], 9)
    return u0, kw, extras
