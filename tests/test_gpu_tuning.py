"""Launch-shape tuning: every supported shape gives the same march, bit for
bit (the per-column and per-plane arithmetic does not depend on the shape),
and the autotuner returns a supported shape whose run still matches."""
import numpy as np
import pytest

import scenarios as S
from gpu_helpers import solver_params

pytestmark = pytest.mark.gpu

KEYS = ["field", "pnp", "ppp", "pI", "pIloss", "zaxis", "pax"]


def _case(shape, flux="kt"):
    kw = dict(S.BASE, fluxScheme=flux, useFreqWeightedBoundary=True, useSuperAbsorbing=True,
              boundaryProfile="wendland", propDist=3 * S.BASE["dZmin"])
    u0 = S.seeded_field(shape, seed=21, amp=3e6).astype(np.float32)
    return solver_params(kw), u0


def _run(plan, u0, dz, steps=3):
    plan.run(u0, steps * dz, dz)
    return plan.outputs()


@pytest.mark.parametrize("shape,flux", [((32, 128, 1024), "kt"), ((64, 128, 256), "rusanov"),
                                        ((32, 64, 512), "kt"), ((256, 256, 256), "kt")])
def test_every_shape_gives_the_same_march(shape, flux):
    from angularspectrum_heterogeneous_gb300 import Plan
    from angularspectrum_heterogeneous_gb300.solver import initial_step
    params, u0 = _case(shape, flux)
    dz = initial_step(u0, params)
    plan = Plan(shape, params, kt_cfl_target=0.4 if flux == "kt" else 0.0)
    try:
        plan.set_operators(0, dz)
        ref = _run(plan, u0, dz)
        default = plan.get_tuning()
        shapes = [dict(t_cols_flux=8, t_cols_plain=8, t_cols_stats=8, xy_clusters=0,
                       xy_clusters_closing=2, xy_sync=1, xy_bulk=1),
                  dict(t_cols_flux=16, t_cols_plain=16, t_cols_stats=16, xy_clusters=3,
                       xy_clusters_closing=0, xy_sync=2, xy_bulk=3, t_prefetch=2, xy_rows=1),
                  dict(t_cols_flux=0, t_cols_plain=0, t_cols_stats=0, xy_clusters=0,
                       xy_clusters_closing=0, xy_sync=2),
                  dict(t_cols_flux=0, t_cols_plain=0, t_cols_stats=0, xy_clusters=5,
                       xy_clusters_closing=0, xy_sync=3, xy_bulk=2, xy_rows=2),
                  dict(t_cols_flux=0, t_cols_plain=0, t_cols_stats=0, xy_clusters=0,
                       xy_clusters_closing=0, xy_sync=3, xy_rows=1)]
        for tun in shapes:
            plan.set_tuning(tun)
            got = plan.get_tuning()
            for k in ("t_cols_flux", "t_cols_plain", "t_cols_stats"):
                assert tun[k] == 0 or got[k] == tun[k]
            assert got["xy_sync"] == (tun["xy_sync"] if default["xy_sync"] else 0)
            out = _run(plan, u0, dz)
            for k, a, b in zip(KEYS, ref, out):
                assert np.array_equal(a, b), (tun, k)
        plan.set_tuning(dict(t_cols_flux=0, t_cols_plain=0, t_cols_stats=0, xy_clusters=0,
                             xy_clusters_closing=0, xy_sync=0))
        assert plan.get_tuning() == default
    finally:
        plan.close()


def test_unsupported_shape_is_rejected():
    from angularspectrum_heterogeneous_gb300 import Plan
    from angularspectrum_heterogeneous_gb300._lib import ASGError
    params, u0 = _case((32, 36, 256))
    plan = Plan((32, 36, 256), params)
    try:
        with pytest.raises(ASGError):
            plan.set_tuning(dict(t_cols_flux=16, t_cols_plain=0, t_cols_stats=0, xy_clusters=0))
        with pytest.raises(ASGError):
            plan.set_tuning(dict(t_cols_flux=0, t_cols_plain=12, t_cols_stats=0, xy_clusters=0))
        with pytest.raises(ASGError):
            plan.set_tuning(dict(t_cols_flux=0, t_cols_plain=0, t_cols_stats=0, xy_clusters=99))
        with pytest.raises(ASGError):
            plan.set_tuning(dict(t_cols_flux=0, t_cols_plain=0, t_cols_stats=0, xy_clusters=0,
                                 xy_rows=3))
    finally:
        plan.close()


@pytest.mark.parametrize("sync", [2, 3])
def test_group_barrier_wait_runs_out_and_the_plan_recovers(sync):
    """The counter barriers of the cooperative plane kernels (plain, and split
    into arrive and wait) are bounded: with a target no group reaches, every
    wait gives up after a second, the run ends with ASG_ERR_TIMEOUT, and the
    next run (normal targets) matches the earlier one bit for bit."""
    from angularspectrum_heterogeneous_gb300 import Plan
    from angularspectrum_heterogeneous_gb300._lib import ASGError
    from angularspectrum_heterogeneous_gb300.solver import initial_step
    shape = (256, 256, 128)
    params, u0 = _case(shape)
    dz = initial_step(u0, params)
    plan = Plan(shape, params)
    try:
        plan.set_operators(0, dz)
        plan.set_tuning(dict(t_cols_flux=0, t_cols_plain=0, t_cols_stats=0, xy_clusters=0,
                             xy_clusters_closing=0, xy_sync=sync))
        assert plan.get_tuning()["xy_sync"] == sync
        ref = _run(plan, u0, dz, steps=2)
        _lib_check(plan, 1)
        with pytest.raises(ASGError) as e:
            _run(plan, u0, dz, steps=2)
        assert e.value.code == -5  # ASG_ERR_TIMEOUT
        _lib_check(plan, 0)
        out = _run(plan, u0, dz, steps=2)
        for k, a, b in zip(KEYS, ref, out):
            assert np.array_equal(a, b), k
    finally:
        plan.close()


def _lib_check(plan, skew):
    from angularspectrum_heterogeneous_gb300 import _lib
    _lib.check(plan.lib.asg_debug_set_barrier_skew(plan.h, skew))


def test_autotune_picks_a_supported_shape_and_keeps_the_result():
    from angularspectrum_heterogeneous_gb300 import Plan
    from angularspectrum_heterogeneous_gb300 import solver
    from angularspectrum_heterogeneous_gb300.solver import initial_step
    shape = (64, 128, 512)
    params, u0 = _case(shape)
    dz = initial_step(u0, params)
    plan = Plan(shape, params)
    try:
        plan.set_operators(0, dz)
        ref = _run(plan, u0, dz)
        chosen = plan.autotune(u0, dz, steps=2)
        assert chosen["t_cols_flux"] in (8, 16) and chosen["t_cols_plain"] in (8, 16)
        assert 0 <= chosen["xy_clusters"] <= 64 and 0 <= chosen["xy_clusters_closing"] <= 64
        assert solver.TUNING_CACHE[plan.tuning_key] == chosen
        out = _run(plan, u0, dz)
        for k, a, b in zip(KEYS, ref, out):
            assert np.array_equal(a, b), k
    finally:
        plan.close()
    # a new plan with the same grid and options starts from the tuned shapes
    plan2 = Plan(shape, params)
    try:
        got = plan2.get_tuning()
        for k in ("t_cols_flux", "t_cols_plain", "t_cols_stats"):
            assert got[k] == chosen[k]
    finally:
        plan2.close()


@pytest.mark.parametrize("shape,flux", [((64, 128, 256), "kt"), ((16, 14, 64), "rusanov")])
def test_graph_replay_matches_eager_steps(shape, flux):
    """Regular steps replayed from the captured step graph give the eager march
    bit for bit, and a second run reuses the graph."""
    from angularspectrum_heterogeneous_gb300 import Plan
    from angularspectrum_heterogeneous_gb300.solver import initial_step
    params, u0 = _case(shape, flux)
    dz = initial_step(u0, params)
    plan = Plan(shape, params)
    try:
        plan.set_operators(0, dz)
        plan.set_graphs(False)
        eager = _run(plan, u0, dz, steps=7)
        plan.set_graphs(True)
        for _ in range(2):
            out = _run(plan, u0, dz, steps=7)
            for k, a, b in zip(KEYS, eager, out):
                assert np.array_equal(a, b), k
        launches = sum(v[1] for v in plan.kernel_stats().values())
        plan.set_graphs(False)
        _run(plan, u0, dz, steps=7)
        assert launches == sum(v[1] for v in plan.kernel_stats().values())
    finally:
        plan.close()
