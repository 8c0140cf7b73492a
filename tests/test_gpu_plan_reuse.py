"""angular_spectrum_solve keeps the plan of its last call (grid and parameters
unchanged, no screens or sources) for the next one: the reused plan gives the
same outputs bit for bit as a fresh one, a failed call drops it, and calls with
screens keep nothing."""
import numpy as np
import pytest

import scenarios as S
from gpu_helpers import KEYS, solver_params

pytestmark = pytest.mark.gpu

SHAPE = (64, 64, 128)


def _field(peak, seed):
    kw = dict(S.BASE)
    kw.update(fluxScheme="kt", useFreqWeightedBoundary=True, useSuperAbsorbing=True,
              propDist=5 * kw["dZmin"])
    nX, nY, nT = SHAPE
    u0 = S.piston_field(nX, nY, nT, kw["dX"], kw["dY"], kw["dT"], kw["f0"], peak,
                        radius=0.35 * nX * kw["dX"], focus=8e-3)
    rng = np.random.default_rng(seed)
    u0 = u0 * (1.0 + 0.01 * rng.standard_normal(u0.shape))
    return u0.astype(np.float32), kw


def test_reused_plan_matches_a_fresh_one():
    from angularspectrum_heterogeneous_gb300 import angular_spectrum_solve, release_cached_plan
    from angularspectrum_heterogeneous_gb300 import solver as SV
    ua, kw = _field(2e6, 1)
    ub, _ = _field(3e6, 2)
    prm = solver_params(kw, {})
    release_cached_plan()
    SV.KEEP_LAST_PLAN = True
    try:
        angular_spectrum_solve(ua, prm, verbose=False)
        kept = SV._LAST_PLAN["plan"]
        assert kept is not None
        reused = angular_spectrum_solve(ub, prm, verbose=False)
        assert SV._LAST_PLAN["plan"] is kept
        release_cached_plan()
        assert SV._LAST_PLAN["plan"] is None
        SV.KEEP_LAST_PLAN = False
        fresh = angular_spectrum_solve(ub, prm, verbose=False)
        assert SV._LAST_PLAN["plan"] is None
    finally:
        SV.KEEP_LAST_PLAN = True
    for k, a, b in zip(KEYS, reused, fresh):
        assert np.array_equal(a, b), k


def test_failed_call_drops_the_plan_and_screens_keep_none():
    from angularspectrum_heterogeneous_gb300 import (StabilityError, angular_spectrum_solve,
                                                     release_cached_plan)
    from angularspectrum_heterogeneous_gb300 import solver as SV
    ua, kw = _field(2e6, 3)
    prm = solver_params(kw, {})
    release_cached_plan()
    ref = angular_spectrum_solve(ua, prm, verbose=False)
    assert SV._LAST_PLAN["plan"] is not None
    with pytest.raises(StabilityError):
        angular_spectrum_solve(ua * 300.0, prm, verbose=False)
    assert SV._LAST_PLAN["plan"] is None
    again = angular_spectrum_solve(ua, prm, verbose=False)
    for k, a, b in zip(KEYS, ref, again):
        assert np.array_equal(a, b), k
    # with phase screens nothing is kept
    nX, nY, _ = SHAPE
    ex = {"phaseScreens": S._screens(nX, nY, 5, [2.0e-4], [False])}
    angular_spectrum_solve(ua, solver_params(kw, ex), verbose=False)
    assert SV._LAST_PLAN["plan"] is None
    release_cached_plan()
