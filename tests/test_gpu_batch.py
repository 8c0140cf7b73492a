"""Batched march of independent instances with uneven grids, step counts and
options: every instance equals its own single-instance run bit for bit, and
one instance is checked against the FP64 oracle."""
import numpy as np
import pytest

import oracle.asm_oracle as O
import scenarios as S
from gpu_helpers import KEYS, TOL, oracle_params, rel, solver_params

pytestmark = pytest.mark.gpu

# (shape, options, peak, steps(+ fraction for a partial last step), screens/sources)
INSTANCES = [
    ((64, 128, 256), dict(fluxScheme="kt", useFreqWeightedBoundary=True, useSuperAbsorbing=True),
     3e6, 7.0, False),
    ((32, 64, 128), dict(fluxScheme="rusanov", boundaryProfile="wendland"), 2e6, 5.5, False),
    ((64, 64, 512), dict(fluxScheme="kt"), 6e6, 4.0, False),
    ((48, 40, 96), dict(useSplitStep=False, alpha0=-1.0), 1e6, 6.0, True),
    ((128, 128, 256), dict(fluxScheme="kt", useSuperAbsorbing=True), 5e5, 3.25, False),
    # 512-wide planes: a cooperative launch alone, thread-block clusters in the batch
    ((512, 512, 128), dict(fluxScheme="kt", useFreqWeightedBoundary=True,
                           useSuperAbsorbing=True), 2e6, 3.0, False),
]


def _inputs(shape, opts, p0, nsteps, extras, seed):
    nX, nY, nT = shape
    kw = dict(S.BASE)
    kw.update(opts)
    kw["propDist"] = nsteps * kw["dZmin"]
    u0 = S.piston_field(nX, nY, nT, kw["dX"], kw["dY"], kw["dT"], kw["f0"], p0,
                        radius=0.35 * nX * kw["dX"], focus=8e-3)
    ex = {}
    if extras:
        ex["phaseScreens"] = S._screens(nX, nY, seed, [3.0e-4, 9.0e-4], [False, True])
        ex["sourcePlanes"] = S._sources(nX, nY, nT, kw["dT"], kw["f0"], [5.0e-4], seed)
    return u0.astype(np.float32), kw, ex


def test_batch_matches_single_runs_and_oracle():
    from angularspectrum_heterogeneous_gb300 import angular_spectrum_solve, solve_batch
    fields, params, singles = [], [], []
    for j, (shape, opts, p0, nsteps, extras) in enumerate(INSTANCES):
        u0, kw, ex = _inputs(shape, opts, p0, nsteps, extras, 7 + j)
        prm = solver_params(kw, ex)
        fields.append(u0)
        params.append(prm)
        singles.append(angular_spectrum_solve(u0, prm, verbose=False))
    outs, ms = solve_batch(fields, params, return_timing=True)
    assert ms > 0
    # the lone 512-wide plan ran as a cooperative launch (split-phase barriers)
    from angularspectrum_heterogeneous_gb300 import Plan
    pl = Plan(fields[-1].shape, params[-1])
    try:
        assert pl.get_tuning()["xy_sync"] == 3
    finally:
        pl.close()
    for j, (a, b) in enumerate(zip(outs, singles)):
        for k, x, y in zip(KEYS, a, b):
            assert x.shape == y.shape, (j, k)
            assert np.array_equal(x, y), (j, k)
    # instance 0 (the 512x512x1024 workload's options) against the FP64 oracle
    u0, kw, ex = _inputs(*INSTANCES[0][:4], INSTANCES[0][4], 7)
    ref = O.solve(u0, oracle_params(kw, ex), "fp64")
    for k, a, r in zip(KEYS, outs[0], ref):
        if k == "zaxis":
            np.testing.assert_array_equal(a, r)
        else:
            assert rel(a, r) < TOL[k], (k, rel(a, r))


def test_batch_without_graphs_is_identical():
    from angularspectrum_heterogeneous_gb300.solver import Batch, _prepared_plan
    plans, us, dzs, props = [], [], [], []
    try:
        for j, (shape, opts, p0, nsteps, extras) in enumerate(INSTANCES[:3]):
            u0, kw, ex = _inputs(shape, opts, p0, nsteps, extras, 7 + j)
            prm = solver_params(kw, ex)
            plan, dz, _ = _prepared_plan(u0, prm)
            plans.append(plan)
            us.append(u0)
            dzs.append(dz)
            props.append(prm.propDist)
        b = Batch(plans)
        try:
            b.run(us, props, dzs)
            with_graphs = [p.outputs() for p in plans]
            b.set_graphs(False)
            b.run(us, props, dzs)
            without = [p.outputs() for p in plans]
        finally:
            b.close()
        for x, y in zip(with_graphs, without):
            for k, a, c in zip(KEYS, x, y):
                assert np.array_equal(a, c), k
    finally:
        for p in plans:
            p.close()


def test_batch_reports_the_failing_instance():
    from angularspectrum_heterogeneous_gb300 import StabilityError, solve_batch
    shape, opts, p0, nsteps, extras = INSTANCES[1]
    u0, kw, ex = _inputs(shape, opts, p0, nsteps, extras, 3)
    good = solver_params(kw, ex)
    with pytest.raises(StabilityError) as e:
        solve_batch([u0, u0 * 200.0], [good, solver_params(kw, ex)])
    assert "instance 1" in str(e.value)
