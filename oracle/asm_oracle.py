"""CPU oracle for the angular-spectrum march -- TEST INFRASTRUCTURE ONLY.

This module is a numpy restatement of the reference solver's hot path
(``angular_spectrum_solver.py`` of pinton-lab/angularspectrum_heterogeneous).
It exists to check the CUDA implementation and to time a CPU baseline.  Only
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py`` (its CPU-baseline
legs) may import it, and only as the checker; the product package never does.

Parity of this restatement is pinned against fixtures produced by running the
reference module itself (``tests/golden/make_golden.py``); see
``tests/test_oracle_golden.py``.

Precision modes
---------------
``fp32``  mirrors the reference as shipped: operators are built in float64 and
          cast to complex64/float32 where the reference casts them
          (``:1342-1369``), the field starts as float32 (``:1408``) and then
          follows numpy's promotion rules.  As in the reference, a
          super-absorbing step or a phase screen promotes the field to float64
          (``:219-227`` builds its coefficient from the float64 ``rfftfreq``).
``fp64``  every float32/complex64 cast becomes float64/complex128: the FP64
          oracle.

Divergence from the reference (deliberate, documented): when the stability
test at ``:1420`` fails, the reference restarts from z=0 with a step that can
never fall below ``dZmin`` (``:1423-1424``), so it restarts forever.  The
oracle raises :class:`StabilityError` instead, as the product does.

FFT backend: ``numpy.fft`` (pocketfft, single thread; the reference's CPU
arithmetic) or ``scipy.fft`` with ``workers`` threads for the timed CPU
baseline.  Select with :func:`set_fft_backend`.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass
from typing import Optional

import numpy as np

# ---------------------------------------------------------------------------
# FFT backend
# ---------------------------------------------------------------------------
_FFT = {"mod": np.fft, "workers": None}


def set_fft_backend(name: str = "numpy", workers: Optional[int] = None):
    """Use numpy's pocketfft ("numpy") or scipy.fft with ``workers`` threads."""
    if name == "numpy":
        _FFT["mod"], _FFT["workers"] = np.fft, None
    elif name == "scipy":
        import scipy.fft as sf
        _FFT["mod"], _FFT["workers"] = sf, (workers or os.cpu_count())
    else:
        raise ValueError(name)


def _f(name, *a, **k):
    mod = _FFT["mod"]
    if _FFT["workers"] is not None and name not in ("fftshift", "ifftshift"):
        k["workers"] = _FFT["workers"]
    return getattr(mod, name)(*a, **k)


class StabilityError(RuntimeError):
    """Raised where the reference would restart forever (``:1420-1439``)."""


# ---------------------------------------------------------------------------
# Parameters (angular_spectrum_solver.py:35-76)
# ---------------------------------------------------------------------------
@dataclass
class OracleParams:
    dX: float = 0.0
    dY: float = 0.0
    dT: float = 0.0
    c0: float = 1500.0
    rho0: float = 1000.0
    beta: float = 3.5
    alpha0: float = 0.5
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
    boundaryProfile: str = "quadratic"
    useFreqWeightedBoundary: bool = False
    useSuperAbsorbing: bool = False
    superAbsorbingStrength: float = 0.8
    fluxScheme: str = "rusanov"
    useObliquityCorrection: bool = True
    useNonlinearityObliquity: bool = False
    phaseScreens: object = None
    sourcePlanes: object = None
    # Extension, not a reference field: > 0 sub-cycles the KT step per (x, y)
    # column at this CFL target (flux_kt_percolumn), the semantics of the GPU
    # path's per-column mode and of the plain fallback of its learned stage.
    kt_cfl_target: float = 0.0


# ---------------------------------------------------------------------------
# 1-D tapers (:82-110) and boundary weights (:275-284)
# ---------------------------------------------------------------------------
def _edge_coordinate(N: int, n: int) -> np.ndarray:
    """s in [0,1]: 1 at the outermost sample, falling linearly to 0 over n samples.

    Both tapers of the reference (``:82-110``) and the super-absorbing weights
    (``:275-284``) use this coordinate: s=(n-1-i)/n on the low edge and
    s=(i-(N-n-1))/n on the high edge; the high edge is written second, so it
    wins where the two overlap (n > N/2).
    """
    s = np.full(N, np.nan)
    i = np.arange(N)
    lo = i < n
    s[lo] = (n - i[lo] - 1) / n
    hi = i >= N - n
    s[hi] = (i[hi] - (N - n - 1)) / n
    return s


def taper_quadratic(N: int, n: int) -> np.ndarray:
    """``ablvec`` (:82-91): 1 - s^2 in the edge bands, 1 inside."""
    s = _edge_coordinate(N, n)
    return np.where(np.isnan(s), 1.0, 1.0 - np.nan_to_num(s) ** 2)


def taper_wendland(N: int, n: int) -> np.ndarray:
    """``ablvec_wendland`` (:94-110): 1-10s^3+15s^4-6s^5, clipped to [0,1]."""
    s = np.nan_to_num(_edge_coordinate(N, n))
    v = 1.0 - 10 * s ** 3 + 15 * s ** 4 - 6 * s ** 5
    v = np.where(np.isnan(_edge_coordinate(N, n)), 1.0, v)
    return np.clip(v, 0.0, 1.0)


def boundary_weights(N: int, n: int) -> np.ndarray:
    """``_make_boundary_weights`` (:275-284): s in the edge bands, 0 inside; float32."""
    s = _edge_coordinate(N, n)
    return np.where(np.isnan(s), 0.0, s).astype(np.float32)


def band_width(n: int, factor: float) -> int:
    """``max(round(n*factor), 1)`` with Python's round-half-even (:121-123)."""
    return max(round(n * factor), 1)


def boundary_layer(nX, nY, nT, factor, profile, enabled=True):
    """(abl, abl_half) float32 (X,Y,T) tables: ``precalculate_abl`` /
    ``precalculate_identity_abl`` (:116-138).  The product is formed in float64
    and rounded to float32; the half step is sqrt of the float32 value."""
    if not enabled:
        one = np.ones((nX, nY, nT), np.float32)
        return one, one.copy()
    vec = taper_wendland if profile == "wendland" else taper_quadratic
    vx = vec(nX, band_width(nX, factor))
    vy = vec(nY, band_width(nY, factor))
    vt = vec(nT, band_width(nT, factor))
    abl = ((vx[:, None] * vy[None, :])[:, :, None] * vt[None, None, :]).astype(np.float32)
    return abl, np.sqrt(abl)


def freq_weighted_mask(nX, nY, nT, dT, f0, factor, profile):
    """``precalculate_abl_freq`` (:144-179): abl_xy ** clip(f0/max(f_m,f_1), .1, 10)."""
    vec = taper_wendland if profile == "wendland" else taper_quadratic
    axy = np.outer(vec(nX, band_width(nX, factor)), vec(nY, band_width(nY, factor)))
    freqs = np.fft.rfftfreq(nT, dT)
    fmin = freqs[1] if len(freqs) > 1 else 1.0
    expo = np.clip(f0 / np.maximum(freqs, fmin), 0.1, 10.0)
    return (axy[:, :, None] ** expo[None, None, :]).astype(np.float32)


# ---------------------------------------------------------------------------
# Wavenumber grids (:403-408, :488-494)
# ---------------------------------------------------------------------------
def centered_grid(n: int, d: float, c: float = 1.0) -> np.ndarray:
    """The reference's centred grid: linspace(0,n-1,n)/(n-1)/d*2pi/c minus its mean.

    Its spacing is 2pi/((n-1) d), not the FFT spacing 2pi/(n d) -- kept as is.
    """
    g = np.linspace(0, n - 1, n) / (n - 1) / d * 2 * np.pi
    if c != 1.0:
        g = g / c
    return g - np.mean(g)


def transverse_kk(nX, nY, dX, dY):
    kx = centered_grid(nX, dX)
    ky = centered_grid(nY, dY)
    return kx[:, None] ** 2 + ky[None, :] ** 2


def kfilter_mask(nX, nY, nT, dX, dY, dZ, dT, c0, adaptive, thr, strength):
    """Cosine k-space taper of ``precalculate_mas`` (:410-433)."""
    kt = centered_grid(nT, dT, c0)
    kk = transverse_kk(nX, nY, dX, dY)
    kmax = min(np.pi / dX, np.pi / dY)
    nz = kt[kt != 0]
    lam = c0 / np.mean(np.abs(nz)) if nz.size else c0 / (1.0 / dT)
    if adaptive:
        cutoff = thr * (1 + strength * (dZ / lam) * 5)
        ktmax = min(kmax * (1 - cutoff), kmax * 0.95)
        kstart = ktmax * 0.8
    else:
        ktmax = kmax * 0.95
        kstart = ktmax * 0.9
    kr = np.sqrt(kk)
    m = np.ones_like(kr)
    band = (kr > kstart) & (kr <= ktmax)
    if np.any(band):
        m[band] = 0.5 * (1 + np.cos(np.pi * (kr[band] - kstart) / (ktmax - kstart)))
    m[kr > ktmax] = 0.0
    return m


def propagator(nX, nY, nT, dX, dY, dZ, dT, c0, adaptive=False, thr=0.05, strength=0.7,
               half=False):
    """Analytic-signal propagator of ``precalculate_mas`` (:396-462), complex128,
    fftshift-centred in all three axes.

    exp(i dz (k - kz)) for kk < k^2 (kz = sqrt(k^2-kk)), exp(dz (i k - sqrt(kk-k^2)))
    otherwise, with dz = dZ (or dZ/2 when ``half``); times the k-filter, which
    is always sized from the full dZ (``:416``, also for the half step at
    ``:446-450``); the first nT//2+1 shifted t-bins (negative frequencies and
    DC) zeroed and the rest doubled.
    """
    kt = centered_grid(nT, dT, c0)
    kk = transverse_kk(nX, nY, dX, dY)
    mask = kfilter_mask(nX, nY, nT, dX, dY, dZ, dT, c0, adaptive, thr, strength)
    dz = dZ / 2 if half else dZ
    k = kt[None, None, :]
    kk3 = kk[:, :, None]
    prop = kk3 < k ** 2
    h_prop = np.exp(dz * (1j * k - 1j * np.sqrt((k ** 2 - kk3) + 0j)))
    h_ev = np.exp(dz * (1j * k - np.sqrt((kk3 - k ** 2) + 0j)))
    H = np.where(prop, h_prop, h_ev) * mask[:, :, None]
    H[:, :, : nT // 2 + 1] = 0
    return H * 2


# ---------------------------------------------------------------------------
# Attenuation / Kramers-Kronig dispersion (:468-592)
# ---------------------------------------------------------------------------
def alpha_terms(alpha0, f0, nT, dT, pw, water):
    """alpha(f), alphaStar(f) on f = m/(nT dT), m=0..nT-1 (:523-535, :555-574)."""
    f = np.arange(nT) / (nT * dT)
    if water:
        conv = alpha0 / 1e12 * 1e2 / (20 * np.log10(np.e))
        alpha = conv * f ** 2
        a0 = (conv / (2 * np.pi) ** 2) * np.tan(np.pi) * ((2 * np.pi * f) - (2 * np.pi * f0))
        astar = 2 * np.pi * a0 * f
    else:
        fs = f.copy()
        fs[0] = fs[1] / 2
        conv = alpha0 / (1e6 ** pw) * 1e2 / (20 * np.log10(np.e))
        alpha = conv * f ** pw
        if pw % 2 == 1:
            a0 = (-2 * conv / ((2 * np.pi) ** pw) / np.pi) * (np.log(2 * np.pi * fs)
                                                               - np.log(2 * np.pi * f0))
        else:
            a0 = (conv / (2 * np.pi) ** pw) * np.tan(np.pi * pw / 2) * \
                 ((2 * np.pi * f) ** (pw - 1) - (2 * np.pi * f0) ** (pw - 1))
        astar = 2 * np.pi * a0 * f
    astar[0] = 0
    return alpha, astar


def atten_filter(alpha, astar, nX, nY, nT, dX, dY, dZ, dT, c0, scale, obliquity, clip_negative):
    """``_build_oblique_atten_filter`` (:468-520), complex128 (X,Y,nT)."""
    kk = transverse_kk(nX, nY, dX, dY)[:, :, None]
    km = (2 * np.pi * np.arange(nT) / (nT * dT) / c0)[None, None, :]
    base = -(alpha + 1j * astar)[None, None, :] * dZ * scale
    if obliquity:
        kzsq = km ** 2 - kk
        prop = kzsq > 0
        kz = np.where(prop, np.maximum(np.sqrt(np.maximum(kzsq, 0.0)), np.abs(km) * 1e-6), 1.0)
        obl = np.where(prop, np.abs(km) / kz, 0.0)
        out = np.where(prop, np.exp(base * obl), 1.0 + 0j)
    else:
        out = np.broadcast_to(np.exp(base), (nX, nY, nT)).astype(np.complex128)
    out = np.array(out, dtype=np.complex128)
    out[:, :, 0] = 1.0          # DC stays unity (km == 0 is skipped in the reference)
    if clip_negative:
        out = np.where(np.real(out) < 0, 0, out)
    return out


def atten_filters(p: OracleParams, nX, nY, nT, dZ):
    """(full, half) filters as ``_build_operators`` chooses them (:1316-1328)."""
    water = p.alpha0 < 0
    a0 = 2.17e-3 if water else p.alpha0
    alpha, astar = alpha_terms(a0, p.f0, nT, p.dT, p.attenPow, water)
    args = (alpha, astar, nX, nY, nT, p.dX, p.dY, dZ, p.dT, p.c0)
    full = atten_filter(*args, 1.0, p.useObliquityCorrection, water)
    half = atten_filter(*args, 0.5, p.useObliquityCorrection, water)
    return full, half


def obliquity_map(nX, nY, nT, dX, dY, dT, c0):
    """``precalculate_obliquity_map`` (:598-627): k/kz on rfft bins, float32."""
    kk = transverse_kk(nX, nY, dX, dY)[:, :, None]
    nf = nT // 2 + 1
    km = (2 * np.pi * np.arange(nf) / (nT * dT) / c0)[None, None, :]
    kzsq = km ** 2 - kk
    prop = kzsq > 0
    kz = np.where(prop, np.maximum(np.sqrt(np.maximum(kzsq, 0.0)), np.abs(km) * 1e-6), 1.0)
    out = np.where(prop, np.abs(km) / kz, 0.0).astype(np.float32)
    out[:, :, 0] = 0.0
    return out


# ---------------------------------------------------------------------------
# Step operators (:185-272, :352-390, :630-685)
# ---------------------------------------------------------------------------
def diffraction_step(u, HH, abl):
    """``_angular_spectrum_step`` (:649-655)."""
    U = _f("fftshift", _f("fftn", u))
    return np.real(_f("ifftn", _f("ifftshift", U * HH))) * abl


def attenuation_step(u, afilt_rfft):
    """``_attenuation_step`` (:667-685): afilt is (X,Y,nT//2+1), xy-centred."""
    nT = u.shape[2]
    F = _f("fftshift", _f("fft2", _f("rfft", u, axis=2), axes=(0, 1)), axes=(0, 1))
    F = _f("ifft2", _f("ifftshift", F * afilt_rfft, axes=(0, 1)), axes=(0, 1))
    return _f("irfft", F, n=nT, axis=2).real


def freq_weighted_step(u, mask):
    """``_freq_weighted_boundary_step`` (:658-664)."""
    return _f("irfft", _f("rfft", u, axis=2) * mask, n=u.shape[2], axis=2)


def _edge_gradient(F, d, axis):
    """Central differences, one-sided at both ends (:232-235, :254-257)."""
    G = np.zeros_like(F)
    sl = [slice(None)] * 3

    def S(a, b):
        s = list(sl)
        s[axis] = slice(a, b)
        return tuple(s)

    G[S(1, -1)] = (F[S(2, None)] - F[S(None, -2)]) / (2 * d)
    G[S(0, 1)] = (F[S(1, 2)] - F[S(0, 1)]) / d
    G[S(-1, None)] = (F[S(-1, None)] - F[S(-2, -1)]) / d
    return G


def super_absorbing_step(u, wx, wy, dX, dY, dT, c0, strength):
    """``_super_absorbing_step`` (:185-272): Engquist-Majda incoming-wave removal
    in (x, y, omega); x edges first, then y edges on the x-corrected spectrum."""
    nX, nY, nT = u.shape
    F = _f("rfft", u, axis=2)
    nf = F.shape[2]
    w = 2.0 * np.pi * np.fft.rfftfreq(nT, dT)
    wmin = 2.0 * np.pi * np.fft.rfftfreq(nT, dT)[1] if nf > 1 else 1.0
    ok = np.abs(w) > 0.5 * wmin
    coeff = np.where(ok, -1j * c0 / np.where(ok, w, 1.0), 0.0 + 0j)[None, None, :]
    for axis, wv, d, n in ((0, wx, dX, nX), (1, wy, dY, nY)):
        G = _edge_gradient(F, d, axis)
        lo = (np.arange(n) < n // 2) * wv
        hi = (np.arange(n) >= n // 2) * wv
        shp = [1, 1, 1]
        shp[axis] = n
        lo = lo.reshape(shp)
        hi = hi.reshape(shp)
        p_lo = 0.5 * (F + coeff * G)
        p_hi = 0.5 * (F - coeff * G)
        F = F - strength * lo * p_lo
        F = F - strength * hi * p_hi
    return _f("irfft", F, n=nT, axis=2)


def phase_screen_step(u, phase, f0_bin, amp=None):
    """``_apply_phase_screen`` (:352-390): F * exp(-i phase m/f0b) * clip(amp)^(m/f0b)."""
    nT = u.shape[2]
    F = _f("rfft", u, axis=2)
    nf = F.shape[2]
    fs = np.arange(nf, dtype=phase.dtype) / np.maximum(f0_bin, 1.0)
    F = F * np.exp(-1j * phase[:, :, None] * fs[None, None, :])
    if amp is not None:
        F = F * np.power(np.clip(amp, 1e-6, 1.0)[:, :, None], fs[None, None, :])
    return _f("irfft", F, n=nT, axis=2)


def beam_obliquity(u, obl):
    """``_beam_obliquity_scalar`` (:630-643): power-weighted mean of k/kz."""
    F = _f("rfft", u, axis=2)
    F = _f("fftshift", _f("fft2", F, axes=(0, 1)), axes=(0, 1))
    P = (F.real ** 2 + F.imag ** 2).astype(obl.dtype)
    return np.sum(P * obl) / (np.sum(P * (obl > 0).astype(obl.dtype)) + 1e-30)


# ---------------------------------------------------------------------------
# Burgers fluxes along t (:688-868).  u has t on its last axis.
# ---------------------------------------------------------------------------
def flux_rusanov(u, N, dZ, dT):
    """``_rusanov_flux_standard`` (:688-696): flux -(uL^2+uR^2)/2 - a (uR-uL)."""
    uL, uR = u[..., :-1], u[..., 1:]
    a = np.maximum(np.abs(uL), np.abs(uR))
    fh = -(uL ** 2 + uR ** 2) / 2 - a * (uR - uL)
    out = np.array(u, copy=True)
    out[..., 1:-1] = u[..., 1:-1] + (-N * dZ / dT * (fh[..., 1:] - fh[..., :-1]))
    return out


def flux_rusanov_tvd(u, N, dZ, dT, beta_tvd):
    """``_rusanov_flux_tvd`` (:699-724): flux/4 form times the mean of the
    generalized-minmod limiters of r and 1/r."""
    uL, uR = u[..., :-1], u[..., 1:]
    a = np.maximum(np.abs(uL), np.abs(uR))
    fh = 0.5 * (-0.5 * (uL ** 2 + uR ** 2)) - 0.5 * a * (uR - uL)
    fd = fh[..., 1:] - fh[..., :-1]
    dm = u[..., 1:-1] - u[..., :-2]
    dp = u[..., 2:] - u[..., 1:-1]
    eps = 1e-30
    r = dp / (dm + eps * np.sign(dm + eps))
    ri = dm / (dp + eps * np.sign(dp + eps))

    def lim(x):
        return np.maximum(0.0, np.minimum(np.minimum(beta_tvd * x, 1.0), np.minimum(x, beta_tvd)))

    out = np.array(u, copy=True)
    out[..., 1:-1] = u[..., 1:-1] + (-N * dZ / dT * (0.5 * (lim(r) + lim(ri)) * fd))
    return out


def _minmod2(a, b):
    return np.where(a * b > 0, np.sign(a) * np.minimum(np.abs(a), np.abs(b)), 0.0)


def _minmod3(a, b, c):
    ok = (a * b > 0) & (b * c > 0)
    return np.where(ok, np.sign(a) * np.minimum(np.minimum(np.abs(a), np.abs(b)), np.abs(c)), 0.0)


def kt_rhs(u, N, dT, limiter="mc"):
    """``_kt_rhs`` / ``_kt_rhs_minmod`` (:758-830): MUSCL slopes (MC or minmod),
    one-sided speeds of f'(u)=-u, KT flux with Lax-Friedrichs fallback where
    |a+ - a-| < 1e-14, zero rhs at both ends."""
    dm = u[..., 1:-1] - u[..., :-2]
    dp = u[..., 2:] - u[..., 1:-1]
    if limiter == "mc":
        s_mid = _minmod3(2 * dm, 0.5 * (dm + dp), 2 * dp)
    else:
        s_mid = _minmod2(dm, dp)
    pad = [(0, 0)] * (u.ndim - 1) + [(1, 1)]
    s = np.pad(s_mid, pad)
    um = u[..., :-1] + 0.5 * s[..., :-1]
    up = u[..., 1:] - 0.5 * s[..., 1:]
    ap = np.maximum(np.maximum(-um, -up), 0.0)
    am = np.minimum(np.minimum(-um, -up), 0.0)
    fm = -0.5 * um ** 2
    fp = -0.5 * up ** 2
    den = ap - am
    small = np.abs(den) < 1e-14
    sd = np.where(small, 1.0, den)
    kt = (ap * fm - am * fp - ap * am * (up - um)) / sd
    lf = 0.5 * (fm + fp) - 0.5 * np.maximum(np.abs(um), np.abs(up)) * (up - um)
    fh = np.where(small, lf, kt)
    rhs = np.zeros_like(u)
    rhs[..., 1:-1] = -N / dT * (fh[..., 1:] - fh[..., :-1])
    return rhs


def flux_kt(u, N, dZ, dT, limiter="mc"):
    """``_kt_flux`` / ``_kt_flux_minmod`` (:833-839, :862-868): SSP-RK2."""
    s1 = u + dZ * kt_rhs(u, N, dT, limiter)
    return 0.5 * u + 0.5 * (s1 + dZ * kt_rhs(s1, N, dT, limiter))


def flux_kt_adaptive(u, N, dZ, dT, cfl_target=0.5):
    """``_kt_flux_adaptive`` (:842-859): global-max CFL sub-cycling."""
    umax = float(np.max(np.abs(u)))
    cfl = N * umax * dZ / dT
    if cfl <= cfl_target or umax < 1e-30:
        return flux_kt(u, N, dZ, dT)
    n = int(math.ceil(cfl / cfl_target))
    for _ in range(n):
        u = flux_kt(u, N, dZ / n, dT)
    return u


def flux_kt_percolumn(u, N, dZ, dT, cfl_target=0.5):
    """Per-column sub-cycling: each (x, y) column takes ceil(N max|u_col| dZ/dT /
    cfl_target) SSP-RK2 KT sub-steps (at least one).  With one column this is
    ``flux_kt_adaptive``; it is the oracle of the product's per-column mode."""
    shp = u.shape
    cols = u.reshape(-1, shp[-1])
    out = np.empty_like(cols)
    umax = np.max(np.abs(cols), axis=1)
    nsub = np.ones(cols.shape[0], np.int64)
    for i in range(cols.shape[0]):
        cfl = N * float(umax[i]) * dZ / dT
        if not (cfl <= cfl_target or umax[i] < 1e-30):
            nsub[i] = int(math.ceil(cfl / cfl_target))
    # columns with the same count step together (each column's arithmetic is
    # its own, so this equals stepping them one by one)
    for n in np.unique(nsub):
        sel = np.nonzero(nsub == n)[0]
        c = cols[sel]
        for _ in range(int(n)):
            c = flux_kt(c, N, dZ / int(n), dT)
        out[sel] = c
    return out.reshape(shp)


# ---------------------------------------------------------------------------
# Driver (:1217-1567)
# ---------------------------------------------------------------------------
def _to_rfft(a, nT):
    return None if a is None else a[:, :, : nT // 2 + 1]


def solve(initial_field, p: OracleParams, precision="fp32", per_step_callback=None,
          max_steps_hint=None):
    """``angular_spectrum_solve`` (:1217-1567), returning the same 7-tuple.

    TOF extraction (``:1387-1397, :1538-1545``) is not part of this path: its
    module is absent from the reference tree.
    """
    rdt = np.float64 if precision == "fp64" else np.float32
    cdt = np.complex128 if precision == "fp64" else np.complex64
    nX, nY, nT = initial_field.shape
    c0 = p.c0
    N = p.beta / (2 * c0 ** 3 * p.rho0)
    maxamp = np.max(np.abs(initial_field))
    dZ = min(p.stabilityRecoveryFactor * p.dT / (maxamp * N + 1e-30), p.dZmin) \
        if maxamp > 0 else p.dZmin
    dZ = max(dZ, p.dZmin)

    def build(dz):
        HH = propagator(nX, nY, nT, p.dX, p.dY, dz, p.dT, c0, p.useAdaptiveFiltering,
                        p.freqFilterThreshold, p.adaptiveFilterStrength)
        HHh = propagator(nX, nY, nT, p.dX, p.dY, dz, p.dT, c0, p.useAdaptiveFiltering,
                         p.freqFilterThreshold, p.adaptiveFilterStrength, half=True) \
            if p.useSplitStep else None
        abl, ablh = boundary_layer(nX, nY, nT, p.boundaryFactor, p.boundaryProfile,
                                   p.useBoundaryLayer)
        af, afh = atten_filters(p, nX, nY, nT, dz)
        ops = dict(HH=HH.astype(cdt), abl=abl.astype(rdt),
                   afilt=_to_rfft(af, nT).astype(cdt))
        if p.useSplitStep:
            ops.update(HH_half=HHh.astype(cdt), abl_half=ablh.astype(rdt),
                       afilt_half=_to_rfft(afh, nT).astype(cdt))
        return ops

    ops = build(dZ)
    fw = freq_weighted_mask(nX, nY, nT, p.dT, p.f0, p.boundaryFactor, p.boundaryProfile) \
        .astype(rdt) if p.useFreqWeightedBoundary else None
    if p.useSuperAbsorbing:
        wx = boundary_weights(nX, band_width(nX, p.boundaryFactor)).astype(rdt)
        wy = boundary_weights(nY, band_width(nY, p.boundaryFactor)).astype(rdt)
    obl = obliquity_map(nX, nY, nT, p.dX, p.dY, p.dT, c0).astype(rdt) \
        if p.useNonlinearityObliquity else None
    f0_bin = p.f0 / (1.0 / (nT * p.dT))

    nmax = int(np.ceil(p.propDist / dZ)) + 100
    pnp = np.zeros((nX, nY, nmax), np.float32)
    ppp = np.zeros_like(pnp)
    pI = np.zeros_like(pnp)
    pIl = np.zeros_like(pnp)
    pax = np.zeros((nT, nmax), np.float32)

    u = np.array(initial_field, dtype=rdt)
    zvec = []
    cc = 0
    while sum(zvec) < p.propDist - 1e-15:
        dzs = min(dZ, p.propDist - sum(zvec))
        umax = np.max(np.abs(u))
        if N * dzs / p.dT * umax > p.stabilityThreshold:
            raise StabilityError(
                f"stability criterion violated at step {cc}: N*dZ/dT*max|p| = "
                f"{N * dzs / p.dT * umax:.4g} > {p.stabilityThreshold}; the step cannot "
                f"shrink below dZmin={p.dZmin}")
        Ib = np.sum(u ** 2, axis=2)
        so = ops if abs(dzs - dZ) <= 1e-15 else build(dzs)

        def Neff(v):
            return N * beam_obliquity(v, obl) if obl is not None else N

        if p.useSplitStep:
            u = attenuation_step(u, so["afilt_half"])
            u = diffraction_step(u, so["HH_half"], so["abl_half"])
            Nn = Neff(u)
            if p.fluxScheme == "kt" and p.kt_cfl_target > 0:
                u = flux_kt_percolumn(u, Nn, dzs, p.dT, p.kt_cfl_target)
            elif p.fluxScheme == "kt":
                u = flux_kt(u, Nn, dzs, p.dT)
            elif p.useTVD:
                beta_tvd = max(1.0, 2.0 - p.adaptiveFilterStrength * (dzs / (c0 / p.f0)) * 10)
                u = flux_rusanov_tvd(u, Nn, dzs, p.dT, beta_tvd)
            else:
                u = flux_rusanov(u, Nn, dzs, p.dT)
            u = diffraction_step(u, so["HH_half"], so["abl_half"])
            u = attenuation_step(u, so["afilt_half"])
        else:
            u = diffraction_step(u, so["HH"], so["abl"])
            u = flux_rusanov(u, Neff(u), dzs, p.dT)
            u = attenuation_step(u, so["afilt"])
        if fw is not None:
            u = freq_weighted_step(u, fw)
        if p.useSuperAbsorbing:
            u = super_absorbing_step(u, wx, wy, p.dX, p.dY, p.dT, c0, p.superAbsorbingStrength)
        z = sum(zvec)
        if p.phaseScreens is not None:
            for scr in p.phaseScreens:
                if z < scr[0] <= z + dzs:
                    amp = np.array(scr[2], dtype=rdt) if len(scr) > 2 and scr[2] is not None \
                        else None
                    u = phase_screen_step(u, np.array(scr[1], dtype=rdt), f0_bin, amp)
        if p.sourcePlanes is not None:
            for sz, sf in p.sourcePlanes:
                if z < sz <= z + dzs:
                    u = u + np.array(sf, dtype=rdt)
        Ia = np.sum(u ** 2, axis=2)
        pIl[:, :, cc] = np.maximum(0, Ib - Ia)
        pI[:, :, cc] = Ia
        pnp[:, :, cc] = np.min(u, axis=2)
        ppp[:, :, cc] = np.max(u, axis=2)
        pax[:, cc] = u[nX // 2, nY // 2, :]
        zvec.append(dzs)
        if per_step_callback is not None:
            per_step_callback(cc, sum(zvec), u)
        cc += 1
    return (np.array(u), pnp[:, :, :cc], ppp[:, :, :cc], pI[:, :, :cc], pIl[:, :, :cc],
            np.cumsum(zvec[:cc]), pax[:, :cc])


# ---------------------------------------------------------------------------
# Step-by-step runner with the same arithmetic as solve(): operators are built
# once (untimed) and march steps are timed separately -- the CPU baseline.
# ---------------------------------------------------------------------------
class OracleMarch:
    """March state for timing: ``build()`` then ``step()`` repeatedly.

    Only regular steps (no partial last step, screens or sources); the step
    body is the one of :func:`solve` (``:1413-1536``)."""

    def __init__(self, initial_field, p: OracleParams, precision="fp32"):
        self.p = p
        self.rdt = np.float64 if precision == "fp64" else np.float32
        self.cdt = np.complex128 if precision == "fp64" else np.complex64
        self.u = np.array(initial_field, dtype=self.rdt)
        self.nX, self.nY, self.nT = self.u.shape
        self.N = p.beta / (2 * p.c0 ** 3 * p.rho0)
        self.dz = max(p.dZmin, min(p.stabilityRecoveryFactor * p.dT /
                                   (float(np.max(np.abs(self.u))) * self.N + 1e-30), p.dZmin))

    def build(self):
        p, nX, nY, nT, dz = self.p, self.nX, self.nY, self.nT, self.dz
        nf = nT // 2 + 1
        if p.useSplitStep:
            self.H = propagator(nX, nY, nT, p.dX, p.dY, dz, p.dT, p.c0, p.useAdaptiveFiltering,
                                p.freqFilterThreshold, p.adaptiveFilterStrength,
                                half=True).astype(self.cdt)
            _, ablh = boundary_layer(nX, nY, nT, p.boundaryFactor, p.boundaryProfile,
                                     p.useBoundaryLayer)
            self.abl = ablh.astype(self.rdt)
            _, afh = atten_filters(p, nX, nY, nT, dz)
            self.af = afh[:, :, :nf].astype(self.cdt)
        else:
            self.H = propagator(nX, nY, nT, p.dX, p.dY, dz, p.dT, p.c0, p.useAdaptiveFiltering,
                                p.freqFilterThreshold, p.adaptiveFilterStrength).astype(self.cdt)
            abl, _ = boundary_layer(nX, nY, nT, p.boundaryFactor, p.boundaryProfile,
                                    p.useBoundaryLayer)
            self.abl = abl.astype(self.rdt)
            af, _ = atten_filters(p, nX, nY, nT, dz)
            self.af = af[:, :, :nf].astype(self.cdt)
        self.fw = freq_weighted_mask(nX, nY, nT, p.dT, p.f0, p.boundaryFactor,
                                     p.boundaryProfile).astype(self.rdt) \
            if p.useFreqWeightedBoundary else None
        if p.useSuperAbsorbing:
            self.wx = boundary_weights(nX, band_width(nX, p.boundaryFactor)).astype(self.rdt)
            self.wy = boundary_weights(nY, band_width(nY, p.boundaryFactor)).astype(self.rdt)
        self.Ib = np.sum(self.u ** 2, axis=2)
        return self

    def step(self):
        p, u, dz = self.p, self.u, self.dz
        if p.useSplitStep:
            u = attenuation_step(u, self.af)
            u = diffraction_step(u, self.H, self.abl)
            if p.fluxScheme == "kt":
                u = flux_kt(u, self.N, dz, p.dT)
            elif p.useTVD:
                bt = max(1.0, 2.0 - p.adaptiveFilterStrength * (dz / (p.c0 / p.f0)) * 10)
                u = flux_rusanov_tvd(u, self.N, dz, p.dT, bt)
            else:
                u = flux_rusanov(u, self.N, dz, p.dT)
            u = diffraction_step(u, self.H, self.abl)
            u = attenuation_step(u, self.af)
        else:
            u = diffraction_step(u, self.H, self.abl)
            u = flux_rusanov(u, self.N, dz, p.dT)
            u = attenuation_step(u, self.af)
        if self.fw is not None:
            u = freq_weighted_step(u, self.fw)
        if p.useSuperAbsorbing:
            u = super_absorbing_step(u, self.wx, self.wy, p.dX, p.dY, p.dT, p.c0,
                                     p.superAbsorbingStrength)
        Ia = np.sum(u ** 2, axis=2)
        self.stats = (np.min(u, axis=2), np.max(u, axis=2), Ia, np.maximum(0, self.Ib - Ia),
                      u[self.nX // 2, self.nY // 2, :].copy())
        self.Ib = Ia
        self.u = u
        return u
