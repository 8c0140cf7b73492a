"""Golden fixture of the GPU-scale plain configuration for its first two steps:
512 x 512 x 1024 float32 grid, dX = dY = 1.5e-4 m, dT = 1e-8 s, f0 = 2 MHz,
c0 = 1540, rho0 = 1000, beta = 3.5, alpha0 = 0.5 dB/cm/MHz (y = 1), a 20 mm
piston focused at 60 mm by a quadratic delay, 5-cycle Gaussian burst of
2 MPa; Strang splitting, KT flux, frequency-weighted and super-absorbing
boundaries, dZ = 1e-4 m, propDist = 2e-4 m (two full steps).

The FP64 oracle marches it; the oracle itself is pinned to the reference by
tests/test_oracle_golden.py.  The outputs are stored reduced so that the
fixture stays a few MB: the final field at every 16th x and y (all 1024
samples of those columns), the field of the central row x = 256 restricted
to |y - 256| < 64, pnp/ppp/pI/pIloss of both steps at every 4th x and y,
pax and zaxis.  The GPU test reduces its own outputs the same way.

    python tests/golden/make_c2_steps.py     (about 10 minutes, ~40 GB of RAM)
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import oracle.asm_oracle as O  # noqa: E402
import scenarios as S  # noqa: E402

C2 = dict(dX=1.5e-4, dY=1.5e-4, dT=1e-8, c0=1540.0, rho0=1000.0, beta=3.5, alpha0=0.5,
          attenPow=1.0, f0=2e6, dZmin=1e-4, propDist=2e-4, fluxScheme="kt",
          useFreqWeightedBoundary=True, useSuperAbsorbing=True)
SHAPE = (512, 512, 1024)


def c2_field():
    return S.piston_field(*SHAPE, C2["dX"], C2["dY"], C2["dT"], C2["f0"], 2e6, radius=20e-3,
                          focus=60e-3, ncycles=5)


def reduce_outputs(out):
    field, pnp, ppp, pI, pIloss, zaxis, pax = out
    return dict(zaxis=np.asarray(zaxis, np.float64),
                field_dec=np.ascontiguousarray(field[::16, ::16, :], np.float32),
                field_row=np.ascontiguousarray(field[256, 192:320, :], np.float32),
                pnp=np.ascontiguousarray(pnp[::4, ::4, :], np.float32),
                ppp=np.ascontiguousarray(ppp[::4, ::4, :], np.float32),
                pI=np.ascontiguousarray(pI[::4, ::4, :], np.float32),
                pIloss=np.ascontiguousarray(pIloss[::4, ::4, :], np.float32),
                pax=np.asarray(pax, np.float32))


if __name__ == "__main__":
    O.set_fft_backend("scipy", os.cpu_count())
    t0 = time.time()
    ref = reduce_outputs(O.solve(c2_field(), O.OracleParams(**C2), "fp64"))
    np.savez_compressed(os.path.join(HERE, "c2_steps_fp64.npz"), **ref)
    print(f"done in {time.time() - t0:.0f} s:",
          {k: v.shape for k, v in ref.items()})
