"""Input builders that feed the march: bowl sources and phase/amplitude screens.

These are the reference's host-side constructors, restated (numpy; they run
once per solve):

* :func:`make_bowl_source`        -- ``angular_spectrum_solver.py:971-1077``
* :func:`make_bowl_source_planes` -- ``angular_spectrum_solver.py:1080-1211``
* :func:`generate_phase_screen`   -- ``angular_spectrum_solver.py:290-349``
* :func:`skull_to_phase_screens`  -- ``validate_transcranial.py:166-238``

Outputs have the reference's types and layouts, so they plug into
``SolverParams.sourcePlanes`` / ``phaseScreens`` unchanged.
"""
from __future__ import annotations

from typing import NamedTuple

import numpy as np


class CompactPlane(NamedTuple):
    """A source plane stored as its non-zero columns only: ``cols`` are the
    flat indices x*nY + y of the columns (int32), ``values`` their samples
    (float32, (len(cols), nT)).  Accepted wherever a dense (nX, nY, nT) source
    plane is (``SolverParams.sourcePlanes``, ``Plan.add_source``)."""
    cols: np.ndarray
    values: np.ndarray
    shape: tuple

    def toarray(self):
        nX, nY, nT = self.shape
        out = np.zeros((nX * nY, nT), np.float32)
        out[self.cols] = self.values
        return out.reshape(nX, nY, nT)


def _bowl_geometry(xaxis, yaxis, radius, roc, inner_radius):
    X, Y = np.meshgrid(xaxis, yaxis, indexing="ij")
    r2 = X ** 2 + Y ** 2
    r = np.sqrt(r2)
    aperture = (r2 <= radius ** 2) & (r2 >= inner_radius ** 2)
    depth = roc - np.sqrt(roc ** 2 - np.minimum(r2, roc ** 2 - 1e-20))
    return r2, r, aperture, depth


def _element_delays(delays, r, aperture, radius, inner_radius, n_elements, element_delays):
    """Average the focusing delay over each of n equal-width annuli and add the
    per-element steering delay."""
    if n_elements > 1:
        dr = (radius - inner_radius) / n_elements
        for e in range(n_elements):
            sel = (r >= inner_radius + e * dr) & (r < inner_radius + (e + 1) * dr) & aperture
            if sel.any():
                delays[sel] = delays[sel].mean()
                if element_delays is not None:
                    delays[sel] += np.asarray(element_delays)[e]
    return delays


def _burst(taxis, delays, mask, f0, p0, ncycles, dur):
    w0 = 2 * np.pi * f0
    tt = taxis[None, None, :] - delays[:, :, None]
    env = np.exp(-(1.05 * tt * w0 / (ncycles * np.pi)) ** (2 * dur))
    return mask[:, :, None] * env * np.sin(w0 * tt) * p0


def make_bowl_source(xaxis, yaxis, taxis, f0, c0, p0, radius, roc, ncycles=3, dur=2,
                     inner_radius=0.0, focus=None, element_delays=None, n_elements=1):
    """Bowl (optionally annular, multi-element) projected onto one source plane.

    Per-pixel delay = distance from the bowl surface point (r, z_bowl(r)) to
    the focus (0, 0, focus) / c0, averaged per annulus, inverted so the
    outermost pixels fire first; each pixel carries the Gaussian-windowed burst
    ``exp(-(1.05 (t-d) w0/(ncycles pi))^(2 dur)) sin(w0 (t-d)) p0``.
    Returns float32 (nX, nY, nT).
    """
    focus = roc if focus is None else focus
    r2, r, ap, zb = _bowl_geometry(xaxis, yaxis, radius, roc, inner_radius)
    d = np.zeros_like(r)
    d[ap] = np.sqrt(r2 + (focus - zb) ** 2)[ap] / c0
    d = _element_delays(d, r, ap, radius, inner_radius, n_elements, element_delays)
    d[ap] = d[ap].max() - d[ap]
    return _burst(np.asarray(taxis), d, ap.astype(np.float32), f0, p0, ncycles, dur) \
        .astype(np.float32)


def make_bowl_source_planes(xaxis, yaxis, taxis, f0, c0, p0, radius, roc, dZ, ncycles=3,
                            dur=2, inner_radius=0.0, focus=None, element_delays=None,
                            n_elements=1, compact=False):
    """The bowl sliced along z into ceil(depth/dZ) layers for plane-by-plane
    injection.  Returns ``([(z_mid, float32 (nX,nY,nT)), ...], bowl_depth)``;
    layers without pixels are skipped; a layer's delays are advanced by
    z_bowl/c0, the distance the march has already covered.

    ``compact=True`` (an extension) returns each layer as a
    :class:`CompactPlane` holding only the layer's pixels, the same numbers
    as the dense plane's non-zero columns, without ever forming the dense
    planes (12 GB for a 384 x 384 x 512 grid and a 14.5 mm deep bowl sliced
    every 0.308 mm; its active columns take 114 MB)."""
    focus = roc if focus is None else focus
    r2, r, ap, zb = _bowl_geometry(xaxis, yaxis, radius, roc, inner_radius)
    zb = np.where(ap, zb, 0.0)
    depth = float(np.max(zb[ap]))
    dfull = np.zeros_like(r)
    dfull[ap] = np.sqrt(r2 + (focus - zb) ** 2)[ap] / c0
    dfull = _element_delays(dfull, r, ap, radius, inner_radius, n_elements, element_delays)
    dfull[ap] = dfull[ap].max() - dfull[ap]
    n = max(1, int(np.ceil(depth / dZ)))
    edges = np.linspace(0, depth, n + 1)
    taxis = np.asarray(taxis)
    planes = []
    for i in range(n):
        lo, hi = edges[i], edges[i + 1]
        sel = ap & (zb >= lo) & ((zb <= hi) if i == n - 1 else (zb < hi))
        if not sel.any():
            continue
        if compact:
            flat = np.flatnonzero(sel).astype(np.int32)
            dsel = dfull.reshape(-1)[flat] - zb.reshape(-1)[flat] / c0
            w0 = 2 * np.pi * f0
            tt = taxis[None, :] - dsel[:, None]
            env = np.exp(-(1.05 * tt * w0 / (ncycles * np.pi)) ** (2 * dur))
            vals = (env * np.sin(w0 * tt) * p0).astype(np.float32)
            planes.append((0.5 * (lo + hi),
                           CompactPlane(flat, vals, (len(xaxis), len(yaxis), len(taxis)))))
            continue
        d = dfull.copy()
        d[sel] -= zb[sel] / c0
        d[~sel] = 0.0
        planes.append((0.5 * (lo + hi),
                       _burst(taxis, d, sel.astype(np.float32), f0, p0, ncycles, dur)
                       .astype(np.float32)))
    return planes, depth


def generate_phase_screen(nX, nY, dX, dY, c0, f0, correlation_length, speed_std,
                          thickness=None, seed=None):
    """Gaussian-random-field sound-speed screen.

    White complex noise filtered by sqrt(exp(-k^2 L^2/4)) on the FFT grid, real
    part normalised to ``speed_std``; phase = w0 * thickness * (1/c - 1/c0).
    Returns (phase float32 (nX,nY), c_map float32 (nX,nY)).
    """
    thickness = correlation_length if thickness is None else thickness
    rng = np.random.default_rng(seed)
    kx = np.fft.fftfreq(nX, dX) * 2 * np.pi
    ky = np.fft.fftfreq(nY, dY) * 2 * np.pi
    K2 = kx[:, None] ** 2 + ky[None, :] ** 2
    filt = np.sqrt(np.exp(-K2 * correlation_length ** 2 / 4.0))
    noise = rng.standard_normal((nX, nY)) + 1j * rng.standard_normal((nX, nY))
    dc = np.real(np.fft.ifft2(np.fft.fft2(noise) * filt))
    dc = dc / (np.std(dc) + 1e-30) * speed_std
    cmap = c0 + dc
    phase = 2 * np.pi * f0 * thickness * (1.0 / cmap - 1.0 / c0)
    return phase.astype(np.float32), cmap.astype(np.float32)


def skull_to_phase_screens(c_map, dz_screen, dz_prop, c0, f0, rho_map=None, rho0=1000.0,
                           alpha_bone=8.0, alpha_tissue=0.5):
    """Sound-speed (and density) volume -> list of (z, phase, amplitude) screens.

    Per z-slice: phase = w0 dz (1/c - 1/c0); amplitude = exp(-alpha dz) with
    alpha interpolated between tissue and bone by the bone fraction
    (c - 1540)/(2900 - 1540) (dB/cm/MHz -> Np/m via 0.1151/0.01), times the
    normal-incidence transmission |2Z/(Z+Z0)| when a density map is given.
    Slices with max|phase| <= 1e-6 and min(amp) >= 0.999 are dropped.
    """
    nx, ny, nz = c_map.shape
    w0 = 2 * np.pi * f0
    fmhz = f0 / 1e6
    out = []
    for iz in range(nz):
        c = c_map[:, :, iz]
        phase = w0 * dz_screen * (1.0 / c - 1.0 / c0)
        bone = np.clip((c - 1540.0) / (2900.0 - 1540.0), 0, 1)
        alpha = (alpha_tissue + bone * (alpha_bone - alpha_tissue)) * fmhz * 0.1151 / 0.01
        amp = np.exp(-alpha * dz_screen)
        if rho_map is not None:
            Z = rho_map[:, :, iz] * c
            amp = amp * np.abs(2.0 * Z / (Z + rho0 * c0))
        if np.max(np.abs(phase)) > 1e-6 or np.min(amp) < 0.999:
            out.append((iz * dz_screen, phase.astype(np.float32), amp.astype(np.float32)))
    return out
