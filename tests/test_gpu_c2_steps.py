"""The 512 x 512 x 1024 KT workload itself (KT, frequency-weighted and
super-absorbing boundaries, Strang, its dX, dT, f0 and 2 MPa focused piston)
for its first two full steps on the GPU, against the FP64 oracle's run stored
reduced in tests/golden/c2_steps_fp64.npz by tests/golden/make_c2_steps.py.
This runs exactly the kernel instantiations the benchmark times: 1024-sample
column passes and cooperative plane passes over 512-wide planes."""
import os

import numpy as np
import pytest

from gpu_helpers import TOL, rel, solver_params

pytestmark = pytest.mark.gpu

FIX = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "c2_steps_fp64.npz")


@pytest.mark.skipif(not os.path.exists(FIX), reason="fixture not generated")
def test_workload_two_steps_match_fp64_oracle():
    import make_c2_steps as MC
    from angularspectrum_heterogeneous_gb300 import angular_spectrum_solve
    ref = np.load(FIX)
    got = MC.reduce_outputs(angular_spectrum_solve(MC.c2_field(), solver_params(MC.C2),
                                                   verbose=False))
    np.testing.assert_array_equal(got["zaxis"], ref["zaxis"])
    errs = {k: rel(got[k], ref[k]) for k in got if k != "zaxis"}
    print("\nrel-L2 vs FP64 oracle:", {k: f"{v:.2e}" for k, v in errs.items()})
    tol = {"field_dec": TOL["field"], "field_row": TOL["field"], "pnp": TOL["pnp"],
           "ppp": TOL["ppp"], "pI": TOL["pI"], "pIloss": TOL["pIloss"], "pax": TOL["pax"]}
    for k, e in errs.items():
        assert e < tol[k], (k, errs)
