"""Learned KT corrector: host side of the CUDA network (asg_net_* in the C ABI).

The network maps one coarse KT step of a t-column (scaled by the column's peak)
to the correction that brings it to the fully sub-cycled KT step:

    out = coarse + s * gamma * cfl^3 * net(coarse * N/dT * dz / 0.3)

with s = max|u| of the column entering the step and cfl = N/dT * s * dz its
CFL number.  The input is in CFL units, so the network sees the column's CFL
number.  The difference between one SSP-RK2 KT step and the sub-cycled
step is third order in the CFL number, so the scaled targets are of order one
at every peak; gamma is one constant fitted on the training data.  Below a CFL
number of about 0.1 the difference is at the level of FP32 rounding: those
columns are left out of the loss and take the plain KT step at run time.

Forward and backward run in the library's own kernels (BF16 tensor-core GEMMs
for the 64x64 layers, FP32 accumulation, FP32 master weights, Adam); this
module only orchestrates: parameter initialisation, the training loop over
device batches and the data generation from the plain KT kernel.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

NCH, KT5 = 64, 5
SHAPES = [("W1", (NCH, 1, KT5)), ("b1", (NCH,)), ("W2", (NCH, NCH, KT5)), ("b2", (NCH,)),
          ("W3", (NCH, NCH, KT5)), ("b3", (NCH,)), ("W4", (1, NCH, KT5)), ("b4", (1,))]


def param_count() -> int:
    return int(sum(np.prod(s) for _, s in SHAPES))


def to_dict(theta):
    """Flat parameter vector -> {name: array} with W[out][in][tap] shapes."""
    out, o = {}, 0
    for name, shp in SHAPES:
        n = int(np.prod(shp))
        out[name] = np.asarray(theta[o:o + n], dtype=np.float32).reshape(shp)
        o += n
    return out


def from_dict(d):
    return np.concatenate([np.asarray(d[name], np.float32).reshape(-1) for name, _ in SHAPES])


def init_params(seed: int = 0, last_scale: float = 1e-2):
    """He-style initialisation; the last layer starts small so that the
    untrained correction is close to zero."""
    rng = np.random.default_rng(seed)
    d = {}
    for name, shp in SHAPES:
        if name.startswith("b"):
            d[name] = np.zeros(shp, np.float32)
        else:
            fan_in = shp[1] * shp[2]
            d[name] = (rng.standard_normal(shp) * np.sqrt(2.0 / fan_in)).astype(np.float32)
    d["W4"] *= last_scale
    return from_dict(d)


class Corrector:
    """The network on the current CUDA device."""

    def __init__(self, theta=None, seed: int = 0):
        self.lib = _lib.load()
        h = C.c_void_p()
        _lib.check(self.lib.asg_net_create(C.byref(h)))
        self.h = h
        assert self.lib.asg_net_param_count() == param_count()
        self.set_params(init_params(seed) if theta is None else theta)
        self.gamma = 1.0

    def set_output_scale(self, gamma: float):
        _lib.check(self.lib.asg_net_set_output_scale(self.h, float(gamma)))
        self.gamma = float(gamma)

    def close(self):
        if getattr(self, "h", None):
            self.lib.asg_net_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, theta):
        t = np.ascontiguousarray(theta, dtype=np.float32)
        _lib.check(self.lib.asg_net_set_params(self.h, _lib.fptr(t), t.size))

    def get_params(self):
        t = np.empty(param_count(), np.float32)
        _lib.check(self.lib.asg_net_get_params(self.h, _lib.fptr(t), t.size))
        return t

    def forward(self, x, y=None, stream=None):
        """x: CUDA float32 tensor (ncols, nT) -> y (same shape)."""
        import torch
        assert x.is_cuda and x.dtype == torch.float32 and x.dim() == 2 and x.is_contiguous()
        if y is None:
            y = torch.empty_like(x)
        s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        _lib.check(self.lib.asg_net_forward(self.h, C.c_void_p(x.data_ptr()),
                                            C.c_void_p(y.data_ptr()), x.shape[0], x.shape[1],
                                            C.c_void_p(s)))
        return y

    def train_step(self, x, target, mask, lr: float, want_grad: bool = False):
        """One Adam step (lr > 0) or a gradient evaluation (lr = 0) on a device
        batch; returns the masked MSE loss (and the gradient vector)."""
        import torch
        torch.cuda.synchronize()
        loss = C.c_double(0.0)
        g = np.empty(param_count(), np.float32) if want_grad else None
        _lib.check(self.lib.asg_net_train_step(
            self.h, C.c_void_p(x.data_ptr()), C.c_void_p(target.data_ptr()),
            C.c_void_p(mask.data_ptr()), x.shape[0], x.shape[1], float(lr), C.byref(loss),
            _lib.fptr(g)))
        return (loss.value, g) if want_grad else loss.value


# ---------------------------------------------------------------------------
# training data: (column before, column after the fully sub-cycled KT step)
# ---------------------------------------------------------------------------
MIN_CFL = 0.1  # columns below this CFL number are left out of the loss
CFL_IN = 0.3   # input unit of the network, in CFL units


def _flux_device(cols, out, n_coef, dz, dt, cfl_target, max_sub, flux=_lib.FLUX_KT):
    import torch
    lib = _lib.load()
    _lib.check(lib.asg_flux_columns_device(
        C.c_void_p(cols.data_ptr()), C.c_void_p(out.data_ptr()), cols.shape[0], cols.shape[1],
        flux, float(n_coef), float(dz), float(dt), 1.0, float(cfl_target), int(max_sub),
        C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    if cfl_target > 0.0:
        # a target column capped at max_sub sub-cycles would not be the fully
        # sub-cycled step the network is trained towards
        n, need = C.c_uint(0), C.c_uint(0)
        _lib.check(lib.asg_flux_columns_device_clamped(
            C.c_void_p(torch.cuda.current_stream().cuda_stream), C.byref(n), C.byref(need)))
        if n.value:
            raise _lib.SubcycleCapError(
                -9, f"{n.value} target columns needed up to {need.value} sub-cycles "
                    f"(cap {max_sub})")
    return out


def training_pairs(cols, n_coef, dz, dt, cfl_target, gamma=1.0, max_sub=4096, min_cfl=MIN_CFL):
    """Network input, target and mask of a device batch of columns (ncols, nT):
    x = coarse n_coef/dt dz / 0.3 (CFL units), target = (fine - coarse) /
    (s gamma cfl^3), with coarse one
    KT step of dz, fine the KT step sub-cycled at cfl_target, s = max|u| and
    cfl = n_coef/dt s dz per column; the mask drops the end samples and the
    columns below min_cfl.  Also returns coarse and fine."""
    import torch
    coarse = _flux_device(cols, torch.empty_like(cols), n_coef, dz, dt, 0.0, 1)
    fine = _flux_device(cols, torch.empty_like(cols), n_coef, dz, dt, cfl_target, max_sub)
    s = cols.abs().amax(dim=1, keepdim=True).clamp_min(1e-30)
    cfl = (n_coef / dt * dz) * s
    x = (coarse * (n_coef / dt * dz / CFL_IN)).contiguous()
    target = ((fine - coarse) / (s * gamma * cfl ** 3)).contiguous()
    mask = (cfl >= min_cfl).float().expand_as(cols).contiguous()
    mask[:, 0] = 0.0
    mask[:, -1] = 0.0
    return x, target, mask, coarse, fine


def random_focused_field(grid, rng, dX=1.5e-4, dT=1e-8, focus_range=(15e-3, 40e-3)):
    """One seeded random focused field (peak 0.5-3 MPa, 1-3 MHz, aperture
    radius 0.25-0.4 of the grid width, focus drawn from focus_range, 2-6
    cycles) on an (nX, nY, nT) grid; returns (field, f0)."""
    nX, nY, nT = grid
    x = (np.arange(nX) - (nX - 1) / 2.0) * dX
    y = (np.arange(nY) - (nY - 1) / 2.0) * dX
    t = np.arange(nT) * dT
    t = t - t.mean()
    XX, YY = np.meshgrid(x, y, indexing="ij")
    p0 = rng.uniform(0.5e6, 3e6)
    f0 = rng.uniform(1e6, 3e6)
    radius = rng.uniform(0.25, 0.4) * nX * dX
    focus = rng.uniform(*focus_range)
    ncyc = rng.uniform(2.0, 6.0)
    r2 = XX ** 2 + YY ** 2
    ap = r2 <= radius ** 2
    delay = np.where(ap, r2 / (2 * focus * 1540.0), 0.0)
    delay = np.where(ap, delay - delay[ap].mean(), 0.0)
    w0 = 2 * np.pi * f0
    u0 = np.zeros((nX, nY, nT), np.float32)
    ix, iy = np.nonzero(ap)
    for s0 in range(0, ix.size, 4096):  # aperture columns only, in chunks
        sl = slice(s0, s0 + 4096)
        tt = t[None, :] + delay[ix[sl], iy[sl]][:, None]
        u0[ix[sl], iy[sl], :] = (np.exp(-(1.05 * tt * w0 / (ncyc * np.pi)) ** 4)
                                 * np.sin(w0 * tt) * p0).astype(np.float32)
    return u0, f0


def focused_field_columns(n_fields, grid=(96, 96, 1024), steps=40, seed=0, dX=1.5e-4, dT=1e-8,
                          dz=1e-4, min_frac=0.1):
    """Columns of seeded random focused fields (peak 0.5-3 MPa, 1-3 MHz) after
    `steps` march steps of the plain GPU KT solver: a CUDA tensor (ncols, nT) of
    the columns whose peak exceeds min_frac of the field's peak."""
    import torch
    from .solver import SolverParams, angular_spectrum_solve
    rng = np.random.default_rng(seed)
    nT = grid[2]
    out = []
    for _ in range(n_fields):
        u0, f0 = random_focused_field(grid, rng, dX, dT)
        prm = SolverParams(dX=dX, dY=dX, dT=dT, c0=1540.0, rho0=1000.0, beta=3.5, alpha0=0.5,
                           attenPow=1.0, f0=f0, propDist=steps * dz, dZmin=dz, fluxScheme="kt")
        field = angular_spectrum_solve(u0, prm, verbose=False)[0]
        cols = field.reshape(-1, nT)
        peak = np.abs(cols).max(axis=1)
        keep = cols[peak > min_frac * peak.max()]
        out.append(torch.from_numpy(np.ascontiguousarray(keep)).cuda())
    return torch.cat(out, 0)


def train(net, pool, n_coef, dz, dt, cfl_target, steps=500, batch=256, lr=1e-3, seed=0,
          amp_range=(0.7, 1.5), log_every=0):
    """Train on random batches of the column pool with random peak scaling
    (targets from the plain KT kernel, generated on the fly); the output scale
    gamma is fitted first.  Returns the loss history."""
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    idx = torch.randint(0, pool.shape[0], (min(pool.shape[0], 4 * batch),), device="cuda",
                        generator=g)
    _, t0, m0, _, _ = training_pairs(pool[idx].contiguous(), n_coef, dz, dt, cfl_target)
    gamma = float(((t0 * m0) ** 2).sum().div(m0.sum().clamp_min(1.0)).sqrt().clamp_min(1e-30))
    net.set_output_scale(gamma)
    hist = []
    for it in range(steps):
        idx = torch.randint(0, pool.shape[0], (batch,), device="cuda", generator=g)
        amp = torch.empty((batch, 1), device="cuda").uniform_(*amp_range, generator=g)
        cols = (pool[idx] * amp).contiguous()
        x, target, mask, _, _ = training_pairs(cols, n_coef, dz, dt, cfl_target, gamma)
        cur = lr * 0.5 * (1 + np.cos(np.pi * it / steps))
        hist.append(net.train_step(x, target, mask, cur))
        if log_every and it % log_every == 0:
            print(f"step {it} loss {hist[-1]:.3e}")
    return hist


def learned_flux(net, cols, n_coef, dz, dt, cfl_target, min_subcycles, shock_ratio=0.5,
                 max_subcycles=4096, flux=_lib.FLUX_KT, out=None):
    """The learned KT step on a device batch of columns; returns (out, learned count)."""
    import torch
    out = torch.empty_like(cols) if out is None else out
    lib = _lib.load()
    n = C.c_int(0)
    _lib.check(lib.asg_flux_columns_learned(
        net.h, C.c_void_p(cols.data_ptr()), C.c_void_p(out.data_ptr()), cols.shape[0],
        cols.shape[1], flux, float(n_coef), float(dz), float(dt), float(cfl_target),
        int(max_subcycles), int(min_subcycles), float(shock_ratio), C.byref(n),
        C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    return out, n.value
