"""Host-side 1-D operator vectors (FP64) for one step size.

The reference builds dense (nX, nY, nT) operator tables on the host with
Python loops (``angular_spectrum_solver.py:396-627``) and uploads them.  Here
the host only forms the 1-D ingredients -- the centred wavenumber grids, the
cosine k-filter band, alpha(f) and alphaStar(f), the separable boundary
tapers, the frequency-weighted exponents and the super-absorbing weights --
and the device expands them into its FP64-built multiplier tables.

Every function states the reference lines whose arithmetic it restates.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


def _edge_s(N: int, n: int):
    """Edge coordinate of the reference tapers (``:82-110``, ``:275-284``):
    s=(n-1-i)/n on the low band, s=(i-(N-n-1))/n on the high band (written
    second, so it wins where the bands overlap); NaN inside."""
    s = np.full(N, np.nan)
    i = np.arange(N)
    lo = i < n
    s[lo] = (n - i[lo] - 1) / n
    hi = i >= N - n
    s[hi] = (i[hi] - (N - n - 1)) / n
    return s


def taper(N: int, n: int, profile: str) -> np.ndarray:
    """``ablvec`` (quadratic, ``:82-91``) or ``ablvec_wendland`` (``:94-110``)."""
    s = _edge_s(N, n)
    inside = np.isnan(s)
    s = np.nan_to_num(s)
    if profile == "wendland":
        v = np.clip(1.0 - 10 * s ** 3 + 15 * s ** 4 - 6 * s ** 5, 0.0, 1.0)
    else:
        v = 1.0 - s ** 2
    return np.where(inside, 1.0, v)


def boundary_weights(N: int, n: int) -> np.ndarray:
    """``_make_boundary_weights`` (``:275-284``), rounded to float32 as there."""
    s = _edge_s(N, n)
    return np.where(np.isnan(s), 0.0, s).astype(np.float32).astype(np.float64)


def band(n: int, factor: float) -> int:
    """``max(round(n * factor), 1)`` (``:121-123``)."""
    return max(round(n * factor), 1)


def centred_grid(n: int, d: float, c: float = 1.0) -> np.ndarray:
    """``linspace(0,n-1,n)/(n-1)/d*2pi[/c]`` minus its mean (``:403-408``).

    Spacing 2pi/((n-1) d): the reference's grid, not the FFT grid."""
    g = np.linspace(0, n - 1, n) / (n - 1) / d * 2 * np.pi
    if c != 1.0:
        g = g / c
    return g - np.mean(g)


def kfilter_band(nT, dX, dY, dZ, dT, c0, adaptive, thr, strength):
    """(k_trans_start, k_trans_max) of the cosine k-filter (``:413-425``);
    always sized from the full step dZ, also for the half-step propagator."""
    kt = centred_grid(nT, dT, c0)
    kmax = min(np.pi / dX, np.pi / dY)
    nz = kt[kt != 0]
    lam = c0 / np.mean(np.abs(nz)) if nz.size else c0 / (1.0 / dT)
    if adaptive:
        cutoff = thr * (1 + strength * (dZ / lam) * 5)
        ktmax = min(kmax * (1 - cutoff), kmax * 0.95)
        return ktmax * 0.8, ktmax
    ktmax = kmax * 0.95
    return ktmax * 0.9, ktmax


def alpha_terms(alpha0, f0, nT, dT, pw):
    """alpha(f), alphaStar(f) on f_m = m/(nT dT), m < nT.  alpha0 < 0 selects
    the water model (a0=2.17e-3, f^2, ``:1316-1322``, ``:523-535``), otherwise
    the power law with the log (odd pw) or tan (other pw) Kramers-Kronig term
    (``:555-574``).  Returns (alpha, alphaStar, clip_negative)."""
    f = np.arange(nT) / (nT * dT)
    if alpha0 < 0:
        a0 = 2.17e-3
        conv = a0 / 1e12 * 1e2 / (20 * np.log10(np.e))
        alpha = conv * f ** 2
        s0 = (conv / (2 * np.pi) ** 2) * np.tan(np.pi) * ((2 * np.pi * f) ** 1 - (2 * np.pi * f0) ** 1)
        astar = 2 * np.pi * s0 * f
        astar[0] = 0
        return alpha, astar, True
    fs = f.copy()
    fs[0] = fs[1] / 2
    conv = alpha0 / (1e6 ** pw) * 1e2 / (20 * np.log10(np.e))
    alpha = conv * f ** pw
    if pw % 2 == 1:
        s0 = (-2 * conv / ((2 * np.pi) ** pw) / np.pi) * (np.log(2 * np.pi * fs) - np.log(2 * np.pi * f0))
    else:
        s0 = (conv / (2 * np.pi) ** pw) * np.tan(np.pi * pw / 2) * \
            ((2 * np.pi * f) ** (pw - 1) - (2 * np.pi * f0) ** (pw - 1))
    astar = 2 * np.pi * s0 * f
    astar[0] = 0
    return alpha, astar, False


def freq_weight_exponents(nT, dT, f0):
    """clip(f0 / max(f_m, f_1), 0.1, 10) per rfft bin (``:165-176``)."""
    freqs = np.fft.rfftfreq(nT, dT)
    fmin = freqs[1] if len(freqs) > 1 else 1.0
    return np.clip(f0 / np.maximum(freqs, fmin), 0.1, 10.0)


def beta_tvd(dz, c0, f0, strength):
    """TVD limiter parameter of the driver (``:1465-1466``)."""
    return max(1.0, 2.0 - strength * (dz / (c0 / f0)) * 10)


@dataclass
class StepOperators:
    dz: float
    kx: np.ndarray
    ky: np.ndarray
    kt: np.ndarray
    kfilt_start: float
    kfilt_max: float
    alpha: np.ndarray
    alpha_star: np.ndarray
    atten_obliquity: bool
    atten_clip_negative: bool
    abl_x: np.ndarray
    abl_y: np.ndarray
    abl_t: np.ndarray
    fw_exponent: np.ndarray | None
    fw_taper_x: np.ndarray | None
    fw_taper_y: np.ndarray | None
    sa_wx: np.ndarray | None
    sa_wy: np.ndarray | None
    beta_tvd: float


def step_operators(params, nX, nY, nT, dz) -> StepOperators:
    """All 1-D operator vectors of one step size (``_build_operators``,
    ``:1301-1338``, and the boundary extras of ``_to_jax``, ``:1353-1367``)."""
    p = params
    k0, k1 = kfilter_band(nT, p.dX, p.dY, dz, p.dT, p.c0, p.useAdaptiveFiltering,
                          p.freqFilterThreshold, p.adaptiveFilterStrength)
    alpha, astar, clip = alpha_terms(p.alpha0, p.f0, nT, p.dT, p.attenPow)
    prof = p.boundaryProfile
    if p.useBoundaryLayer:
        ax = taper(nX, band(nX, p.boundaryFactor), prof)
        ay = taper(nY, band(nY, p.boundaryFactor), prof)
        at = taper(nT, band(nT, p.boundaryFactor), prof)
    else:
        ax, ay, at = np.ones(nX), np.ones(nY), np.ones(nT)
    fw = fx = fy = None
    if p.useFreqWeightedBoundary:
        fw = freq_weight_exponents(nT, p.dT, p.f0)
        fx = taper(nX, band(nX, p.boundaryFactor), prof)
        fy = taper(nY, band(nY, p.boundaryFactor), prof)
    wx = wy = None
    if p.useSuperAbsorbing:
        wx = boundary_weights(nX, band(nX, p.boundaryFactor))
        wy = boundary_weights(nY, band(nY, p.boundaryFactor))
    return StepOperators(
        dz=dz, kx=centred_grid(nX, p.dX), ky=centred_grid(nY, p.dY),
        kt=centred_grid(nT, p.dT, p.c0), kfilt_start=k0, kfilt_max=k1,
        alpha=alpha, alpha_star=astar, atten_obliquity=bool(p.useObliquityCorrection),
        atten_clip_negative=clip, abl_x=ax, abl_y=ay, abl_t=at, fw_exponent=fw,
        fw_taper_x=fx, fw_taper_y=fy, sa_wx=wx, sa_wy=wy,
        beta_tvd=beta_tvd(dz, p.c0, p.f0, p.adaptiveFilterStrength))


def step_sequence(prop_dist: float, dz: float):
    """Step sizes of the march, formed exactly as the reference's while loop
    does (``:1413-1415``).  ``sum(zvec)`` is Python's built-in sum, which for
    floats is Neumaier-compensated since CPython 3.12; the C driver
    reproduces that summation (``PySum`` in asg_capi.cu)."""
    zvec = []
    while sum(zvec) < prop_dist - 1e-15:
        zvec.append(min(dz, prop_dist - sum(zvec)))
    return zvec
