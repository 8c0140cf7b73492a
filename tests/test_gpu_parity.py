"""GPU parity: the CUDA march (through the C ABI) against the CPU oracle and
the reference-generated fixtures."""
import os

import numpy as np
import pytest

import oracle.asm_oracle as O
import scenarios as S
from gpu_helpers import KEYS, TOL, oracle_params, rel, solver_params

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")
G32 = np.load(os.path.join(GOLD, "golden_fp32.npz"))
G64 = np.load(os.path.join(GOLD, "golden_fp64.npz"))


@pytest.fixture(scope="module")
def lib():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from angularspectrum_heterogeneous_gb300 import _lib
    return _lib.load()


# ---------------------------------------------------------------------------
# Burgers columns (reference golden columns, odd and tiny lengths)
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("nT", [64, 65, 3, 801])
def test_flux_columns_vs_reference(lib, nT):
    from angularspectrum_heterogeneous_gb300 import _lib
    N = 3.5 / (2 * 1540.0 ** 3 * 1000.0)
    col = G64[f"col_{nT}"].astype(np.float32).reshape(1, nT)
    for dZ, dT in [(1.0e-4, 1.0e-8), (5.0e-4, 2.0e-8)]:
        t = f"{nT}_{dZ:g}_{dT:g}"
        for kind, key, extra in [(_lib.FLUX_RUSANOV, "rus", {}),
                                 (_lib.FLUX_RUSANOV_TVD, "tvd", {"beta_tvd": 1.7}),
                                 (_lib.FLUX_KT, "kt", {}),
                                 (_lib.FLUX_KT_MINMOD, "ktmm", {}),
                                 (_lib.FLUX_KT, "ktad", {"cfl_target": 0.05})]:
            out = _lib.flux_columns(col, kind, N, dZ, dT, **extra)
            ref = G64[f"{key}_{t}"].reshape(1, nT)
            assert rel(out, ref) < 2e-6, (key, t, rel(out, ref))


def test_flux_subcycle_cap_is_reported(lib):
    """A column that needs more sub-cycles than the cap is reported
    (ASG_ERR_SUBCYCLES), not run silently above its CFL target."""
    from angularspectrum_heterogeneous_gb300 import SubcycleCapError, _lib
    N = 3.5 / (2 * 1540.0 ** 3 * 1000.0)
    cols = np.stack([S.seeded_column(256, s) * 6.0 for s in range(4)]).astype(np.float32)
    with pytest.raises(SubcycleCapError):
        _lib.flux_columns(cols, _lib.FLUX_KT, N, 4e-4, 1e-8, cfl_target=1e-3, max_subcycles=2)
    _lib.flux_columns(cols, _lib.FLUX_KT, N, 4e-4, 1e-8, cfl_target=1e-3, max_subcycles=4096)


def test_march_subcycle_cap_is_reported(lib):
    from angularspectrum_heterogeneous_gb300 import Plan, SubcycleCapError
    nX, nY, nT = 32, 64, 128
    kw = dict(S.BASE)
    kw.update(fluxScheme="kt", propDist=3 * kw["dZmin"])
    u0 = S.piston_field(nX, nY, nT, kw["dX"], kw["dY"], kw["dT"], kw["f0"], 8e6,
                        radius=0.35 * nX * kw["dX"], focus=8e-3)
    for cap, raises in [(1, True), (4096, False)]:
        plan = Plan((nX, nY, nT), solver_params(kw), kt_cfl_target=1e-3, kt_max_subcycles=cap)
        try:
            plan.set_operators(0, kw["dZmin"])
            if raises:
                with pytest.raises(SubcycleCapError):
                    plan.run(u0, kw["propDist"], kw["dZmin"])
            else:
                plan.run(u0, kw["propDist"], kw["dZmin"])
        finally:
            plan.close()


def test_flux_per_column_subcycles(lib):
    """Per-column CFL sub-cycling: each column its own sub-step count."""
    from angularspectrum_heterogeneous_gb300 import _lib
    N = 3.5 / (2 * 1540.0 ** 3 * 1000.0)
    rng = np.random.default_rng(3)
    cols = np.stack([S.seeded_column(256, s) * a for s, a in
                     zip(range(16), np.linspace(0.2, 8.0, 16))]).astype(np.float32)
    out = _lib.flux_columns(cols, _lib.FLUX_KT, N, 4e-4, 1e-8, cfl_target=0.5)
    ref = O.flux_kt_percolumn(cols.astype(np.float64), N, 4e-4, 1e-8, 0.5)
    assert rel(out, ref) < 5e-6


# ---------------------------------------------------------------------------
# single step operators: generic kernels (golden fields) and fast kernels
# ---------------------------------------------------------------------------
def _op_case(shape, seed=4):
    nX, nY, nT = shape
    kw = dict(dX=2.0e-4, dY=2.5e-4, dT=3.0e-8, c0=1540.0, rho0=1000.0, alpha0=0.5,
              attenPow=1.0, f0=1e6, dZmin=1e-4, boundaryProfile="wendland",
              useFreqWeightedBoundary=True, useSuperAbsorbing=True,
              useNonlinearityObliquity=True)
    u = S.seeded_field(shape, seed=seed, amp=2e6).astype(np.float32)
    return kw, u


OP_SHAPES = [(8, 10, 16), (7, 9, 15), (32, 64, 128), (64, 128, 256), (96, 96, 192),
             (128, 128, 256), (32, 96, 64), (121, 119, 48)]


@pytest.mark.parametrize("shape", OP_SHAPES)
def test_step_operators(lib, shape):
    from angularspectrum_heterogeneous_gb300 import Plan
    nX, nY, nT = shape
    kw, u = _op_case(shape)
    sp = solver_params(kw)
    plan = Plan(shape, sp)
    dz = 1e-4
    plan.set_operators(0, dz)
    rng = np.random.default_rng(7)
    ph = (rng.standard_normal((nX, nY)) * 1.5).astype(np.float32)
    amp = rng.uniform(0.3, 1.2, (nX, nY)).astype(np.float32)
    plan.add_screen(0.0, ph, amp)
    plan.add_screen(0.0, ph, None)
    u64 = u.astype(np.float64)
    p = oracle_params(kw)
    H = O.propagator(nX, nY, nT, p.dX, p.dY, dz, p.dT, p.c0, True, 0.05, 0.7)
    Hh = O.propagator(nX, nY, nT, p.dX, p.dY, dz, p.dT, p.c0, True, 0.05, 0.7, half=True)
    abl, ablh = O.boundary_layer(nX, nY, nT, 0.2, "wendland")
    A, Ah = O.atten_filters(p, nX, nY, nT, dz)
    nf = nT // 2 + 1
    fw = O.freq_weighted_mask(nX, nY, nT, p.dT, p.f0, 0.2, "wendland").astype(np.float64)
    wx = O.boundary_weights(nX, O.band_width(nX, 0.2)).astype(np.float64)
    wy = O.boundary_weights(nY, O.band_width(nY, 0.2)).astype(np.float64)
    f0b = p.f0 / (1.0 / (nT * p.dT))
    cases = {
        1: O.diffraction_step(u64, H, abl.astype(np.float64)),
        2: O.diffraction_step(u64, Hh, ablh.astype(np.float64)),
        3: O.attenuation_step(u64, A[:, :, :nf]),
        4: O.attenuation_step(u64, Ah[:, :, :nf]),
        5: O.freq_weighted_step(u64, fw),
        6: O.super_absorbing_step(u64, wx, wy, p.dX, p.dY, p.dT, p.c0, 0.8),
    }
    for op, ref in cases.items():
        out = plan.apply_operator(op, u)
        assert rel(out, ref) < 2e-6, (shape, op, rel(out, ref))
    out = plan.apply_operator(7, u, 0)
    assert rel(out, O.phase_screen_step(u64, ph.astype(np.float64), f0b,
                                        amp.astype(np.float64))) < 2e-6
    out = plan.apply_operator(7, u, 1)
    assert rel(out, O.phase_screen_step(u64, ph.astype(np.float64), f0b, None)) < 2e-6
    obl = O.obliquity_map(nX, nY, nT, p.dX, p.dY, p.dT, p.c0).astype(np.float64)
    s = plan.apply_operator(8, u)
    ref = O.beam_obliquity(u64, obl)
    assert abs(s - ref) < 1e-5 * abs(ref)
    plan.close()


# ---------------------------------------------------------------------------
# full solves: every option branch of the reference driver (golden fixtures)
# ---------------------------------------------------------------------------
def _gpu_solve(u0, kw, extras):
    from angularspectrum_heterogeneous_gb300 import angular_spectrum_solve
    return angular_spectrum_solve(u0, solver_params(kw, extras), verbose=False)


@pytest.mark.parametrize("name", list(S.SOLVE_SCENARIOS))
def test_solve_vs_reference_fixtures(lib, name):
    u0, kw, ex = S.build_solve_inputs(name)
    res = _gpu_solve(u0, kw, ex)
    for k, a in zip(KEYS, res):
        r64 = G64[f"solve_{name}_{k}"]
        r32 = G32[f"solve_{name}_{k}"]
        assert a.shape == r64.shape, (k, a.shape, r64.shape)
        if k == "zaxis":
            np.testing.assert_array_equal(a, r64)
            continue
        e = rel(a, r64)
        assert e < TOL[k], (name, k, e, "fp32 ref vs fp64:", rel(r32, r64))


# ---------------------------------------------------------------------------
# full solves on the fast kernels against the oracle run live (FP64)
# ---------------------------------------------------------------------------
C2_OPTS = dict(fluxScheme="kt", useFreqWeightedBoundary=True, useSuperAbsorbing=True,
               dX=1.5e-4, dY=1.5e-4, dT=1e-8, f0=2e6, dZmin=1e-4)

FAST_CASES = {
    # options of the 128x128x256 piston workload on a 64^2 x 128 grid
    "tvd_wendland_64": ((64, 64, 128), dict(fluxScheme="rusanov", boundaryProfile="wendland"),
                        4e6, 12),
    # options of the 512x512x1024 piston workload: KT + freq-weighted + super-absorbing, clusters of 2
    "kt_fw_sa_64x128": ((64, 128, 128), dict(fluxScheme="kt", useFreqWeightedBoundary=True,
                                             useSuperAbsorbing=True), 8e6, 10),
    "lie_water_96": ((96, 96, 192), dict(useSplitStep=False, alpha0=-1.0), 3e6, 8),
    # linear medium (beta = 0): the Burgers step is the identity and is skipped
    "linear_kt_fw_sa_64x128": ((64, 128, 128), dict(beta=0.0, fluxScheme="kt",
                                                    useFreqWeightedBoundary=True,
                                                    useSuperAbsorbing=True), 2e6, 6),
    # planes too large for one CTA's shared memory: generic row and column passes
    # over HBM, the epilogue pass, screens and sources; and the power reduction
    "big_odd_kt_fw_sa": ((121, 119, 64), dict(fluxScheme="kt", useFreqWeightedBoundary=True,
                                              useSuperAbsorbing=True), 4e6, 4,
                         dict(zs=[3.0e-4, 6.0e-4], amp=[False, True]),
                         dict(zs=[5.0e-4])),
    "big_odd_obl": ((129, 127, 48), dict(fluxScheme="kt", useNonlinearityObliquity=True),
                    4e6, 3),
    # 256-wide planes: plane kernels in a cooperative launch with counter barriers
    # (diffraction passes with 8-row CTAs in groups of 16, the closing pass and the
    # beam-obliquity power pass with 16-row CTAs in groups of 8), and the Lie march's
    # combined diffraction-attenuation multiplier on the 8-row kernel
    "kt_fw_sa_256_coop": ((256, 256, 128), dict(fluxScheme="kt", useFreqWeightedBoundary=True,
                                                useSuperAbsorbing=True), 4e6, 2),
    "kt_obl_256_coop": ((256, 256, 128), dict(fluxScheme="kt", useNonlinearityObliquity=True),
                        4e6, 2),
    "lie_water_256_coop": ((256, 256, 128), dict(useSplitStep=False, alpha0=-1.0), 3e6, 2),
    "kt_obl_32x64": ((32, 64, 128), dict(fluxScheme="kt", useNonlinearityObliquity=True),
                     6e6, 8),
    # half-plane (split-x) kernels with the beam-obliquity power pass
    "kt_obl_split_64x128": ((64, 128, 128), dict(fluxScheme="kt", useNonlinearityObliquity=True),
                            6e6, 6),
    # half-plane kernels, Lie, water, screens and sources through the epilogue pass
    "lie_screens_sources_split": ((64, 128, 128), dict(useSplitStep=False, alpha0=-1.0), 2e6, 8,
                                  dict(zs=[3.0e-4, 7.5e-4, 1.1e-3], amp=[False, True, True]),
                                  dict(zs=[1.0e-4, 5.0e-4, 1.6e-3])),
    # closing stage with the fused epilogue (both half-planes per cluster): KT,
    # freq-weighted + super-absorbing, screens and sources, clusters of 4
    "kt_fw_sa_screens_fused_128": ((128, 128, 256), dict(fluxScheme="kt",
                                                         useFreqWeightedBoundary=True,
                                                         useSuperAbsorbing=True), 4e6, 6,
                                   dict(zs=[3.0e-4, 9.0e-4], amp=[False, True]),
                                   dict(zs=[5.0e-4, 1.2e-3])),
    # the 128^2 x 256 piston workload's grid at full size for a few steps
    "c1_grid_tvd_wendland": ((128, 128, 256), dict(fluxScheme="rusanov", boundaryProfile="wendland",
                                                   dX=3.08e-4, dY=3.08e-4, f0=1e6), 4e5, 6),
    # the kernel instantiations of the 512x512x1024 KT workload (KT, freq-weighted,
    # super-absorbing, Strang; its dX, dT and f0):
    # 1024-sample columns (the column passes' 512-point complex plan, 16 columns per block)
    "c2_columns_32x128x1024": ((32, 128, 1024), C2_OPTS, 2e6, 8),
    # 512-wide planes: cooperative groups of 16 CTAs over 256-row half-planes
    "c2_planes_512x512x128": ((512, 512, 128), C2_OPTS, 2e6, 2),
    # 384-wide planes: cooperative groups of 12 CTAs
    "c2_planes_384x384x64": ((384, 384, 64), C2_OPTS, 2e6, 3),
}


@pytest.mark.parametrize("name", list(FAST_CASES))
def test_fast_solve_vs_oracle(lib, name):
    shape, kwx, p0, nsteps = FAST_CASES[name][:4]
    nX, nY, nT = shape
    kw = dict(S.BASE)
    kw.update(kwx)
    kw["propDist"] = nsteps * kw["dZmin"]
    u0 = S.piston_field(nX, nY, nT, kw["dX"], kw["dY"], kw["dT"], kw["f0"], p0,
                        radius=0.35 * nX * kw["dX"], focus=8e-3)
    ex = {}
    if len(FAST_CASES[name]) > 4:
        scr, src = FAST_CASES[name][4:6]
        ex["phaseScreens"] = S._screens(nX, nY, 5, scr["zs"], scr["amp"])
        ex["sourcePlanes"] = S._sources(nX, nY, nT, kw["dT"], kw["f0"], src["zs"], 9)
    res = _gpu_solve(u0, kw, ex)
    ref = O.solve(u0, oracle_params(kw, ex), "fp64")
    for k, a, r in zip(KEYS, res, ref):
        if k == "zaxis":
            np.testing.assert_array_equal(a, r)
            continue
        assert rel(a, r) < TOL[k], (name, k, rel(a, r))


def test_stability_violation_raises(lib):
    from angularspectrum_heterogeneous_gb300 import StabilityError
    u0, kw, _ = S.build_solve_inputs("strang_tvd_wendland")
    with pytest.raises(StabilityError):
        _gpu_solve(u0 * 100.0, kw, {})


def test_nan_input_is_rejected(lib):
    from angularspectrum_heterogeneous_gb300 import ASGError
    u0, kw, _ = S.build_solve_inputs("strang_tvd_wendland")
    u0 = u0.copy()
    u0[3, 4, 5] = np.nan
    with pytest.raises(ASGError) as e:
        _gpu_solve(u0, kw, {})
    assert e.value.code == -3


def test_callback_sees_each_step(lib):
    import torch
    from angularspectrum_heterogeneous_gb300 import angular_spectrum_solve
    u0, kw, _ = S.build_solve_inputs("strang_tvd_wendland")
    seen = []

    def cb(cc, z, field):
        assert isinstance(field, torch.Tensor) and field.is_cuda
        seen.append((cc, z, float(field.abs().max())))

    res = angular_spectrum_solve(u0, solver_params(kw), verbose=False, per_step_callback=cb)
    assert [s[0] for s in seen] == list(range(len(res[5])))
    zv = []
    for d in np.diff(np.concatenate([[0.0], res[5]])):
        zv.append(d)
    assert abs(seen[-1][1] - res[5][-1]) < 1e-15
    assert abs(seen[-1][2] - np.abs(res[0]).max()) <= 1e-6 * np.abs(res[0]).max()
