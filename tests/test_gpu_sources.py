"""Compact source planes: a bowl given as its active columns only
(``make_bowl_source_planes(..., compact=True)`` into ``asg_add_source_compact``)
marches exactly like the same bowl given as dense planes, and the compact entry
point rejects columns outside the grid or given twice."""
import numpy as np
import pytest

import angularspectrum_heterogeneous_gb300 as A
from gpu_helpers import solver_params

pytestmark = pytest.mark.gpu

KEYS = ["field", "pnp", "ppp", "pI", "pIloss", "zaxis", "pax"]


def _bowl_case(compact):
    nX, nY, nT = 64, 48, 256
    dX, dT, f0 = 3.08e-4, 4e-8, 1e6
    x = (np.arange(nX) - nX / 2) * dX
    y = (np.arange(nY) - nY / 2) * dX
    t = (np.arange(nT) - nT / 2) * dT
    planes, depth = A.make_bowl_source_planes(
        x, y, t, f0, 1540.0, 4e5, 6.5e-3, 20e-3, dX, inner_radius=2e-3, focus=15e-3,
        n_elements=2, compact=compact)
    kw = dict(dX=dX, dY=dX, dT=dT, c0=1540.0, rho0=1000.0, beta=3.5, alpha0=0.5,
              attenPow=1.0, f0=f0, dZmin=dX, propDist=depth + 4 * dX, fluxScheme="kt",
              useFreqWeightedBoundary=True, useSuperAbsorbing=True)
    return np.zeros((nX, nY, nT), np.float32), solver_params(kw, {"sourcePlanes": planes}), planes


def test_compact_bowl_marches_like_dense_bowl():
    u0, pd, dense = _bowl_case(False)
    _, pc, comp = _bowl_case(True)
    assert len(dense) >= 3 and all(isinstance(p, A.CompactPlane) for _, p in comp)
    assert sum(p.values.size for _, p in comp) < sum(p.size for _, p in dense) // 3
    rd = A.angular_spectrum_solve(u0, pd, verbose=False)
    rc = A.angular_spectrum_solve(u0, pc, verbose=False)
    assert np.abs(rd[0]).max() > 1e4  # the bowl's burst reached the grid
    for k, a, b in zip(KEYS, rd, rc):
        assert np.array_equal(a, b), k


def test_compact_entry_rejects_bad_columns():
    from angularspectrum_heterogeneous_gb300 import Plan
    from angularspectrum_heterogeneous_gb300._lib import ASGError
    u0, pd, _ = _bowl_case(False)
    nX, nY, nT = u0.shape
    plan = Plan(u0.shape, pd)
    try:
        vals = np.ones((2, nT), np.float32)
        for cols in ([0, nX * nY], [-1, 3], [5, 5]):
            with pytest.raises(ASGError):
                plan.add_source(1e-3, A.CompactPlane(np.array(cols, np.int32), vals, u0.shape))
        plan.add_source(1e-3, A.CompactPlane(np.array([0, nX * nY - 1], np.int32), vals,
                                             u0.shape))
    finally:
        plan.close()


# the transcranial-bowl workload scaled down to a 64 x 64 x 128 grid: a 3-element
# bowl (radius 8 mm, roc 16 mm) and a 1-2 mm shell at z = 3.5-5.5 mm
SMALL_TIPS = dict(grid=(64, 64, 128), radius=8e-3, roc=16e-3, inner=3.5e-3, n_elements=3,
                  focus=10e-3, shell_z=(3.5e-3, 5.5e-3), shell_th=(1e-3, 2e-3),
                  shell_roc=16e-3, prop=8e-3)


def test_transcranial_bowl_vs_oracle():
    import scenarios as S
    import oracle.asm_oracle as O
    from gpu_helpers import TOL, oracle_params, rel
    u0, kw, screens, planes = S.tips_inputs(A, compact=True, **SMALL_TIPS)
    _, _, _, dense = S.tips_inputs(A, compact=False, **SMALL_TIPS)
    assert len(screens) >= 4 and len(planes) >= 4
    res = A.angular_spectrum_solve(u0, solver_params(kw, {"sourcePlanes": planes,
                                                          "phaseScreens": screens}),
                                   verbose=False)
    ref = O.solve(u0, oracle_params(kw, {"sourcePlanes": dense, "phaseScreens": screens}),
                  "fp64")
    for k, a, r in zip(KEYS, res, ref):
        if k == "zaxis":
            np.testing.assert_array_equal(a, r)
            continue
        assert rel(a, r) < TOL[k], (k, rel(a, r))
