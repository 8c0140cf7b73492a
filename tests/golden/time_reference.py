"""Times the reference module itself (angular_spectrum_solver.py, imported
through the numpy stand-in for ``jax`` of make_golden.py, FP32 as shipped)
beside the oracle port of it, on the same host cores and the same sample: the
central 128 x 128 x 1024 sub-grid of the 512 x 512 x 1024 KT workload
(freq-weighted and super-absorbing boundaries, dZ = 1e-4 m), march steps
timed through the per-step callback, operator build and the first step
excluded.  The reference cannot travel to the GPU machine (its location is
local), so this records how far the port's timing, which the benchmark's CPU
arm reports, is from the reference's own code.

    python tests/golden/time_reference.py --reference-dir DIR [--steps 3]
"""
import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import make_golden as MG  # noqa: E402
import oracle.asm_oracle as O  # noqa: E402
import scenarios as S  # noqa: E402

GRID = (128, 128, 1024)
KW = dict(dX=1.5e-4, dY=1.5e-4, dT=1e-8, c0=1540.0, rho0=1000.0, beta=3.5, alpha0=0.5,
          attenPow=1.0, f0=2e6, dZmin=1e-4, fluxScheme="kt", useFreqWeightedBoundary=True,
          useSuperAbsorbing=True)


def field():
    return S.piston_field(*GRID, 1.5e-4, 1.5e-4, 1e-8, 2e6, 2e6, radius=20e-3, focus=60e-3,
                          ncycles=5)


def time_reference(ref_dir, steps):
    ref = MG.load_reference(ref_dir, fp64=False)
    ref.jnp = sys.modules["jax.numpy"]
    stamps = []
    p = ref.SolverParams(**dict(KW, propDist=(steps + 1) * KW["dZmin"]))
    ref.angular_spectrum_solve(field(), p, verbose=False,
                               per_step_callback=lambda *a: stamps.append(time.perf_counter()))
    dts = np.diff(stamps)  # step 1 onwards (step 0 carries the operator build)
    return float(np.median(np.prod(GRID) / dts))


def time_port(steps, threads):
    if threads > 1:
        O.set_fft_backend("scipy", threads)
    p = O.OracleParams(**dict(KW, propDist=(steps + 1) * KW["dZmin"]))
    m = O.OracleMarch(field(), p, "fp32").build()
    m.step()
    rates = []
    for _ in range(steps):
        t0 = time.perf_counter()
        m.step()
        rates.append(np.prod(GRID) / (time.perf_counter() - t0))
    O.set_fft_backend("numpy")
    return float(np.median(rates))


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference-dir", default=os.environ.get("ASG_REFERENCE_DIR"))
    ap.add_argument("--steps", type=int, default=3)
    a = ap.parse_args()
    if not a.reference_dir:
        ap.error("give --reference-dir or set ASG_REFERENCE_DIR")
    r = time_reference(a.reference_dir, a.steps)
    p1 = time_port(a.steps, 1)
    pn = time_port(a.steps, os.cpu_count())
    print(f"cores {os.cpu_count()}: reference module (numpy FFT, 1 thread) {r / 1e6:.2f} M "
          f"voxel-steps/s; oracle port numpy FFT {p1 / 1e6:.2f} M; oracle port scipy.fft "
          f"x{os.cpu_count()} {pn / 1e6:.2f} M")
