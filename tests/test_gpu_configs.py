"""The full CPU-runnable configuration (128 x 128 x 256, all 260 steps of
0.25 mm to 65 mm) on the GPU against the reference's own FP32 run of it and
against the FP64 oracle's, both stored reduced in tests/golden/c1_full_fp64.npz
by tests/golden/make_c1_full.py."""
import os

import numpy as np
import pytest

from gpu_helpers import rel, solver_params

pytestmark = pytest.mark.gpu

FIX = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "c1_full_fp64.npz")


@pytest.mark.skipif(not os.path.exists(FIX), reason="fixture not generated")
def test_full_cpu_config_matches_reference_and_fp64():
    import make_c1_full as MC
    from angularspectrum_heterogeneous_gb300 import angular_spectrum_solve
    ref = np.load(FIX)
    out = angular_spectrum_solve(MC.c1_field(), solver_params(MC.C1), verbose=False)
    got = MC.reduce_outputs(out)
    np.testing.assert_array_equal(got["zaxis"], ref["zaxis"])
    assert int(got["focal_step"]) == int(ref["focal_step"])
    keys = [k for k in got if k not in ("zaxis", "focal_step")]
    vs32 = {k: rel(got[k], ref["fp32_" + k]) for k in keys}
    vs64 = {k: rel(got[k], ref[k]) for k in keys}
    ref32 = {k: float(ref["fp32_rel_" + k]) for k in keys}
    print("\nrel-L2 vs reference FP32:", {k: f"{v:.2e}" for k, v in vs32.items()})
    print("rel-L2 vs FP64 oracle:", {k: f"{v:.2e}" for k, v in vs64.items()})
    print("reference FP32 vs FP64:", {k: f"{v:.2e}" for k, v in ref32.items()})
    for k in keys:
        field = k in ("field_dec", "pax")  # pax holds field samples
        # against the reference's own (FP32) run: 1e-4 on the field, 1e-3 on pnp/ppp/pI
        assert vs32[k] < (1e-4 if field else 1e-3), (k, vs32, vs64, ref32)
        # against FP64: within twice the reference's own FP32 distance (and the 1e-3 bar)
        assert vs64[k] < (2.0 * ref32[k] if field else 1e-3), (k, vs32, vs64, ref32)
