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


def _grf(shape, spacing, corr_len, rng):
    """Gaussian random field: white noise filtered by exp(-k^2 L^2 / 4) on the
    FFT grid, scaled to max |g| = 1."""
    noise = rng.standard_normal(shape)
    k2 = 0.0
    for ax, (n, d) in enumerate(zip(shape, spacing)):
        k = np.fft.fftfreq(n, d) * 2 * np.pi
        k2 = k2 + (k ** 2).reshape([-1 if a == ax else 1 for a in range(len(shape))])
    g = np.real(np.fft.ifftn(np.fft.fftn(noise) * np.exp(-k2 * corr_len ** 2 / 4)))
    return g / np.abs(g).max()


def skull_shell(nX, nY, dX, dY, dz, z0=20e-3, z1=29e-3, th_min=5e-3, th_max=9e-3,
                roc=80e-3, c_bone=2800.0, rho_bone=1900.0, porosity=0.1, corr_len=1e-3,
                seed=0):
    """Synthetic curved bone shell as (c, rho) maps on z-slices z0, z0+dz, ..<= z1.

    The shell's near surface is a sphere of radius ``roc`` whose apex is at z0
    on the axis; its thickness varies smoothly between th_min and th_max
    (a 2-D random field of 15 mm correlation length); bone voxels beyond z1
    are cut off.  In bone c = c_bone (1 + porosity g), g a 3-D random field of
    correlation length ``corr_len`` scaled to max |g| = 1 (+-10 % by default),
    rho = rho_bone; elsewhere c = C0, rho = RHO0.  Returns (c, rho) as
    float64 (nX, nY, nz)."""
    rng = np.random.default_rng(seed)
    nz = int(np.floor((z1 - z0) / dz + 1e-9)) + 1
    x = (np.arange(nX) - (nX - 1) / 2.0) * dX
    y = (np.arange(nY) - (nY - 1) / 2.0) * dY
    r2 = x[:, None] ** 2 + y[None, :] ** 2
    sag = roc - np.sqrt(np.maximum(roc ** 2 - r2, 0.0))
    th = th_min + (th_max - th_min) * 0.5 * (1 + _grf((nX, nY), (dX, dY), 15e-3, rng))
    z = z0 + np.arange(nz) * dz
    near = z0 + sag
    bone = (z[None, None, :] >= near[:, :, None]) & (z[None, None, :] < (near + th)[:, :, None])
    bone &= (r2 < roc ** 2)[:, :, None]
    g = _grf((nX, nY, nz), (dX, dY, dz), corr_len, rng)
    c = np.where(bone, c_bone * (1 + porosity * g), C0)
    rho = np.where(bone, rho_bone, RHO0)
    return c, rho


# The transcranial-bowl workload: a TIPS-like annular bowl (radius 46 mm, roc
# 80 mm, inner radius 20.5 mm, 8 elements, 400 kPa, focus 50 mm) sliced into
# source planes, and skull screens of a synthetic shell at z = 20-29 mm, on a
# 384 x 384 x 512 grid with dX = dY = 3.08e-4 m, dT = 4e-8 s, f0 = 1 MHz.  The
# solver options follow the reference's own bowl example
# (``validate_bowl.py:222-290``): linear water (beta 0, alpha0 -1), Strang,
# adaptive filtering, standard Rusanov, Wendland taper with boundaryFactor
# 0.15, frequency-weighted and super-absorbing (strength 0.5) boundaries,
# dZ = dX, propDist 80 mm.
TIPS = dict(grid=(384, 384, 512), dX=3.08e-4, dT=4e-8, f0=1e6, p0=4e5, radius=46e-3,
            roc=80e-3, inner=20.5e-3, n_elements=8, focus=50e-3, shell_z=(20e-3, 29e-3),
            shell_th=(5e-3, 9e-3), shell_roc=80e-3, prop=80e-3)


def tips_inputs(builders, compact=True, **over):
    """(initial field, SolverParams keyword dict, phase screens, source planes)
    of the transcranial-bowl workload; ``over`` replaces entries of TIPS (the
    tests scale it down).  ``builders`` provides make_bowl_source_planes and
    skull_to_phase_screens (the package, or the reference's module)."""
    g = dict(TIPS, **over)
    nX, nY, nT = g["grid"]
    dX, dT, f0 = g["dX"], g["dT"], g["f0"]
    x = np.arange(nX) * dX - (nX - 1) * dX / 2
    y = np.arange(nY) * dX - (nY - 1) * dX / 2
    t = np.arange(nT) * dT - (nT - 1) * dT / 2
    kw = dict(compact=True) if compact else {}
    planes, _ = builders.make_bowl_source_planes(
        x, y, t, f0, C0, g["p0"], g["radius"], g["roc"], dX, focus=g["focus"],
        inner_radius=g["inner"], n_elements=g["n_elements"], **kw)
    z0, z1 = g["shell_z"]
    c, rho = skull_shell(nX, nY, dX, dX, dX, z0, z1, g["shell_th"][0], g["shell_th"][1],
                         g["shell_roc"])
    screens = [(z0 + z, ph, amp) for z, ph, amp in
               builders.skull_to_phase_screens(c, dX, dX, C0, f0, rho_map=rho, rho0=RHO0)]
    first = planes[0][1]
    u0 = first.toarray() if hasattr(first, "toarray") else first
    kw = dict(dX=dX, dY=dX, dT=dT, c0=C0, rho0=RHO0, beta=0.0, alpha0=-1.0, f0=f0,
              propDist=g["prop"], boundaryFactor=0.15, useSplitStep=True,
              useAdaptiveFiltering=True, useTVD=False, dZmin=dX, boundaryProfile="wendland",
              useFreqWeightedBoundary=True, useSuperAbsorbing=True, superAbsorbingStrength=0.5)
    return u0, kw, screens, planes[1:]


BASE = dict(dX=2.5e-4, dY=2.5e-4, dT=4.0e-8, c0=C0, rho0=RHO0, beta=3.5, alpha0=0.5,
            attenPow=1.0, f0=2.0e6, dZmin=2.5e-4, propDist=2.0e-3)

SOLVE_SCENARIOS = {
    # options of the 128x128x256 CPU-runnable piston workload, downscaled: Strang + TVD Rusanov + Wendland
    "strang_tvd_wendland": dict(shape=(16, 16, 48), p0=4e6,
                                kw=dict(fluxScheme="rusanov", boundaryProfile="wendland")),
    # options of the 512x512x1024 piston workload: KT + freq-weighted + super-absorbing
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
