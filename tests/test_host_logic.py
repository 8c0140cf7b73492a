"""Host-side logic of the product package, checked on the CPU against the oracle
and the reference-generated fixtures (no GPU)."""
import os

import numpy as np
import pytest

import angularspectrum_heterogeneous_gb300 as A
from angularspectrum_heterogeneous_gb300 import operators as OP
from angularspectrum_heterogeneous_gb300.solver import SolverParams, flux_kind, initial_step
import oracle.asm_oracle as O

G32 = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_fp32.npz"))


def test_solver_params_defaults_match_reference():
    p = SolverParams()
    q = O.OracleParams()
    # every reference field, with its default; kt_cfl_target is the oracle's
    # extension for the per-column sub-cycled mode (a Plan option here)
    fields = [k for k in q.__dataclass_fields__ if k != "kt_cfl_target"]
    assert sorted(fields) == sorted(p.__dataclass_fields__)
    for k in fields:
        assert getattr(p, k) == getattr(q, k), k


@pytest.mark.parametrize("n,bw", [(16, 3), (17, 4), (5, 1), (128, 26), (7, 5)])
@pytest.mark.parametrize("prof", ["quadratic", "wendland"])
def test_tapers(n, bw, prof):
    ref = O.taper_wendland(n, bw) if prof == "wendland" else O.taper_quadratic(n, bw)
    np.testing.assert_array_equal(OP.taper(n, bw, prof), ref)
    np.testing.assert_array_equal(OP.boundary_weights(n, bw), O.boundary_weights(n, bw))


@pytest.mark.parametrize("pw,a0", [(1.0, 0.5), (2.0, 0.3), (1.5, 0.7), (1.0, -1.0)])
def test_alpha_terms(pw, a0):
    al, ast, clip = OP.alpha_terms(a0, 1e6, 64, 4e-8, pw)
    water = a0 < 0
    al2, ast2 = O.alpha_terms(2.17e-3 if water else a0, 1e6, 64, 4e-8, pw, water)
    np.testing.assert_array_equal(al, al2)
    np.testing.assert_array_equal(ast, ast2)
    assert clip == water


def test_kfilter_band_matches_dense_mask():
    nX, nY, nT, dX, dY, dT, c0, dz = 24, 20, 48, 2.5e-4, 3e-4, 4e-8, 1540.0, 2.5e-4
    for adaptive in (False, True):
        k0, k1 = OP.kfilter_band(nT, dX, dY, dz, dT, c0, adaptive, 0.05, 0.7)
        kk = O.transverse_kk(nX, nY, dX, dY)
        kr = np.sqrt(kk)
        m = np.ones_like(kr)
        band = (kr > k0) & (kr <= k1)
        m[band] = 0.5 * (1 + np.cos(np.pi * (kr[band] - k0) / (k1 - k0)))
        m[kr > k1] = 0
        np.testing.assert_array_equal(m, O.kfilter_mask(nX, nY, nT, dX, dY, dz, dT, c0,
                                                        adaptive, 0.05, 0.7))


def test_step_sequence_matches_reference_loop():
    for prop, dz in [(0.065, 2.5e-4), (0.07, 1e-4), (1.8e-3, 2.5e-4), (2e-3, 2.5e-4)]:
        steps = OP.step_sequence(prop, dz)
        zv = []
        while sum(zv) < prop - 1e-15:
            zv.append(min(dz, prop - sum(zv)))
        assert steps == zv
    assert len(OP.step_sequence(0.065, 2.5e-4)) == 260
    assert len(OP.step_sequence(0.07, 1e-4)) == 700


def test_flux_dispatch():
    assert flux_kind(SolverParams(useSplitStep=False, fluxScheme="kt")) == 1
    assert flux_kind(SolverParams(fluxScheme="kt")) == 3
    assert flux_kind(SolverParams()) == 2
    assert flux_kind(SolverParams(useTVD=False)) == 1


def test_initial_step_is_dzmin():
    u = np.ones((2, 2, 4), np.float32) * 1e6
    assert initial_step(u, SolverParams(dT=4e-8, dZmin=2.5e-4)) == 2.5e-4
    assert initial_step(u * 0, SolverParams(dT=4e-8, dZmin=2.5e-4)) == 2.5e-4


def test_builders_match_reference_fixtures():
    x = (np.arange(24) - 11.5) * 1.0e-3
    y = (np.arange(20) - 9.5) * 1.2e-3
    t = (np.arange(32) - 16) * 8e-8
    planes, depth = A.make_bowl_source_planes(x, y, t, 1e6, 1540.0, 4e5, 10e-3, 25e-3, 1.0e-3,
                                              inner_radius=3e-3, focus=20e-3, n_elements=3)
    np.testing.assert_array_equal(np.array([p[0] for p in planes]), G32["bowl_planes_z"])
    np.testing.assert_array_equal(np.stack([p[1] for p in planes]), G32["bowl_planes_f"])
    assert depth == G32["bowl_depth"]
    b = A.make_bowl_source(x, y, t, 1e6, 1540.0, 4e5, 10e-3, 25e-3, inner_radius=3e-3,
                           focus=20e-3, n_elements=3, element_delays=[0.0, 1e-7, 2e-7])
    np.testing.assert_array_equal(b, G32["bowl_single"])
    ps, cm = A.generate_phase_screen(16, 12, 1e-3, 1.2e-3, 1540.0, 1e6, 3e-3, 40.0,
                                     thickness=2e-3, seed=11)
    np.testing.assert_array_equal(ps, G32["gps_phase"])
    np.testing.assert_array_equal(cm, G32["gps_cmap"])


def test_compact_bowl_planes_equal_the_dense_ones():
    x = (np.arange(24) - 11.5) * 1.0e-3
    y = (np.arange(20) - 9.5) * 1.2e-3
    t = (np.arange(32) - 16) * 8e-8
    kw = dict(inner_radius=3e-3, focus=20e-3, n_elements=3, element_delays=[0.0, 1e-7, 2e-7])
    dense, d1 = A.make_bowl_source_planes(x, y, t, 1e6, 1540.0, 4e5, 10e-3, 25e-3, 1.0e-3, **kw)
    comp, d2 = A.make_bowl_source_planes(x, y, t, 1e6, 1540.0, 4e5, 10e-3, 25e-3, 1.0e-3,
                                         compact=True, **kw)
    assert d1 == d2 and len(dense) == len(comp)
    for (z1, p1), (z2, p2) in zip(dense, comp):
        assert z1 == z2 and isinstance(p2, A.CompactPlane)
        np.testing.assert_array_equal(p2.toarray(), p1)
        nz = np.flatnonzero(np.abs(p1.reshape(-1, 32)).max(axis=1) > 0)
        assert set(nz.tolist()) <= set(p2.cols.tolist())


def test_tof_arguments_follow_reference_errors():
    u = np.zeros((4, 4, 8), np.float32)
    with pytest.raises(ValueError):
        A.angular_spectrum_solve(u, SolverParams(), tof_ref_trace=np.zeros(8))
    with pytest.raises(NotImplementedError):
        A.angular_spectrum_solve(u, SolverParams(), tof_env_ratio=0.5)
