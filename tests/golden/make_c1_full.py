"""Golden fixture of the full CPU-runnable configuration (128 x 128 x 256,
260 steps of 0.25 mm, Strang, TVD-Rusanov, Wendland taper, 400 kPa piston
focused at 50 mm), marched by the FP64 oracle.  The oracle itself is pinned
to the reference by tests/test_oracle_golden.py; this run is too long to
repeat inside the GPU tests, so its outputs are stored reduced:
on-axis pnp/ppp/pI over z, the lateral pnp/ppp/pI slices at the step of peak
on-axis ppp, the final field decimated by 4 in x and y, and zaxis; beside them
the same outputs of the FP32 run (the reference as shipped, which the oracle's
fp32 mode reproduces bit for bit) and their distance from the FP64 run.

    python tests/golden/make_c1_full.py      (about 15 minutes of CPU)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import oracle.asm_oracle as O  # noqa: E402
import scenarios as S  # noqa: E402

C1 = dict(dX=3.08e-4, dY=3.08e-4, dT=4e-8, c0=1540.0, rho0=1000.0, beta=3.5, alpha0=0.5,
          attenPow=1.0, f0=1e6, dZmin=2.5e-4, propDist=0.065, fluxScheme="rusanov",
          boundaryProfile="wendland")
SHAPE = (128, 128, 256)


def c1_field():
    return S.piston_field(*SHAPE, C1["dX"], C1["dY"], C1["dT"], C1["f0"], 4e5, radius=15e-3,
                          focus=50e-3, ncycles=3)


def reduce_outputs(out):
    field, pnp, ppp, pI, pIloss, zaxis, pax = out
    cx, cy = SHAPE[0] // 2, SHAPE[1] // 2
    kf = int(np.argmax(ppp[cx, cy, :]))
    return dict(zaxis=np.asarray(zaxis, np.float64),
                axis_pnp=pnp[cx, cy, :].astype(np.float32),
                axis_ppp=ppp[cx, cy, :].astype(np.float32),
                axis_pI=pI[cx, cy, :].astype(np.float32),
                focal_step=np.int64(kf),
                focal_pnp=pnp[:, :, kf].astype(np.float32),
                focal_ppp=ppp[:, :, kf].astype(np.float32),
                focal_pI=pI[:, :, kf].astype(np.float32),
                field_dec=field[::4, ::4, :].astype(np.float32),
                pax=np.asarray(pax, np.float32))


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


if __name__ == "__main__":
    u0 = c1_field()
    ref = reduce_outputs(O.solve(u0, O.OracleParams(**C1), "fp64"))
    # the reference as shipped (FP32; the oracle's fp32 mode reproduces it bit
    # for bit): its own distance from the FP64 run, stored beside the outputs
    f32 = reduce_outputs(O.solve(u0, O.OracleParams(**C1), "fp32"))
    for k in list(ref):
        if k not in ("zaxis", "focal_step"):
            ref["fp32_rel_" + k] = np.float64(_rel(f32[k], ref[k]))
            ref["fp32_" + k] = f32[k]
    np.savez_compressed(os.path.join(HERE, "c1_full_fp64.npz"), **ref)
    print({k: float(v) for k, v in ref.items() if k.startswith("fp32_rel_")})
