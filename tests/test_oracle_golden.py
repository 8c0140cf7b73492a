"""Pin the CPU oracle to fixtures produced by the reference module itself.

The fixtures (tests/golden/golden_fp32.npz, golden_fp64.npz) were written by
tests/golden/make_golden.py, which runs the reference's own
``angular_spectrum_solver.py`` through a numpy stand-in for jax.  The oracle is
a restatement; these tests show it reproduces the reference bit-for-bit in the
as-shipped float32 mode and to ~1e-13 in the float64 mode.
"""
import os

import numpy as np
import pytest

import oracle.asm_oracle as O
import scenarios as S

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
G32 = np.load(os.path.join(GOLDEN, "golden_fp32.npz"))
G64 = np.load(os.path.join(GOLDEN, "golden_fp64.npz"))


def rel(a, b):
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


SHAPES = [(8, 10, 12), (7, 9, 11)]
dX, dY, dT, c0 = 2.0e-4, 2.5e-4, 3.0e-8, 1540.0


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("ss", [False, True])
@pytest.mark.parametrize("af", [False, True])
def test_propagator(shape, ss, af):
    nX, nY, nT = shape
    tag = f"{nX}x{nY}x{nT}_ss{int(ss)}_af{int(af)}"
    H = O.propagator(nX, nY, nT, dX, dY, 1e-4, dT, c0, af, 0.05, 0.7)
    assert rel(H, G32[f"mas_{tag}_HH"]) < 1e-13
    if ss:
        Hh = O.propagator(nX, nY, nT, dX, dY, 1e-4, dT, c0, af, 0.05, 0.7, half=True)
        assert rel(Hh, G32[f"mas_{tag}_HHhalf"]) < 1e-13


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("prof", ["quadratic", "wendland"])
def test_boundary_layers(shape, prof):
    nX, nY, nT = shape
    tag = f"{nX}x{nY}x{nT}_{prof}"
    abl, ablh = O.boundary_layer(nX, nY, nT, 0.2, prof)
    np.testing.assert_array_equal(abl, G32[f"abl_{tag}"])
    np.testing.assert_array_equal(ablh, G32[f"ablhalf_{tag}"])
    fw = O.freq_weighted_mask(nX, nY, nT, dT, 1e6, 0.2, prof)
    np.testing.assert_allclose(fw, G32[f"ablfreq_{tag}"], rtol=1e-6, atol=1e-7)


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("obl", [False, True])
def test_attenuation_filters(shape, obl):
    nX, nY, nT = shape
    tag = f"{nX}x{nY}x{nT}"
    for water, pw, key in [(True, 1.0, f"adwater_{tag}_obl{int(obl)}")] + \
            [(False, pw, f"adpow_{tag}_pw{pw}_obl{int(obl)}") for pw in (1.0, 2.0, 1.5)]:
        a0 = 2.17e-3 if water else 0.5
        al, ast = O.alpha_terms(a0, 1e6, nT, dT, pw, water)
        for scale, suffix in ((1.0, ""), (0.5, "_half")):
            A = O.atten_filter(al, ast, nX, nY, nT, dX, dY, 1e-4, dT, c0, scale, obl, water)
            assert rel(A, G32[key + suffix]) < 1e-13, key + suffix


@pytest.mark.parametrize("shape", SHAPES)
def test_obliquity_map_and_weights(shape):
    nX, nY, nT = shape
    tag = f"{nX}x{nY}x{nT}"
    np.testing.assert_array_equal(O.obliquity_map(nX, nY, nT, dX, dY, dT, c0),
                                  G32[f"oblmap_{tag}"])
    np.testing.assert_array_equal(O.boundary_weights(nX, 2), G32[f"bdyw_{nX}_2"])


@pytest.mark.parametrize("n,bw", [(16, 3), (17, 4), (5, 1)])
def test_tapers(n, bw):
    np.testing.assert_array_equal(O.taper_quadratic(n, bw), G32[f"ablvec_{n}_{bw}"])
    np.testing.assert_array_equal(O.taper_wendland(n, bw), G32[f"ablvecw_{n}_{bw}"])


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("shape", [(8, 10, 16), (7, 9, 15)])
def test_step_operators(prec, shape):
    G = G32 if prec == "fp32" else G64
    rdt = np.float32 if prec == "fp32" else np.float64
    cdt = np.complex64 if prec == "fp32" else np.complex128
    tol = 1e-6 if prec == "fp32" else 1e-12
    nX, nY, nT = shape
    tag = f"{nX}x{nY}x{nT}"
    u = G[f"in_{tag}"]
    dZ = 1e-4
    Hh = O.propagator(nX, nY, nT, dX, dY, dZ, dT, c0, True, 0.05, 0.7, half=True).astype(cdt)
    _, ablh = O.boundary_layer(nX, nY, nT, 0.2, "wendland")
    assert rel(O.diffraction_step(u, Hh, ablh.astype(rdt)), G[f"diff_{tag}"]) < tol
    al, ast = O.alpha_terms(0.5, 1e6, nT, dT, 1.0, False)
    Ah = O.atten_filter(al, ast, nX, nY, nT, dX, dY, dZ, dT, c0, 0.5, True, False)
    assert rel(O.attenuation_step(u, Ah[:, :, :nT // 2 + 1].astype(cdt)), G[f"atten_{tag}"]) < tol
    fw = O.freq_weighted_mask(nX, nY, nT, dT, 1e6, 0.2, "wendland").astype(rdt)
    assert rel(O.freq_weighted_step(u, fw), G[f"freqw_{tag}"]) < tol
    wx = O.boundary_weights(nX, O.band_width(nX, 0.2)).astype(rdt)
    wy = O.boundary_weights(nY, O.band_width(nY, 0.2)).astype(rdt)
    assert rel(O.super_absorbing_step(u, wx, wy, dX, dY, dT, c0, 0.8), G[f"superabs_{tag}"]) < tol
    ph = G32[f"screen_phase_{tag}"].astype(rdt)
    amp = G32[f"screen_amp_{tag}"].astype(rdt)
    f0b = 1e6 / (1.0 / (nT * dT))
    assert rel(O.phase_screen_step(u, ph, f0b, amp), G[f"screen_{tag}"]) < tol
    assert rel(O.phase_screen_step(u, ph, f0b, None), G[f"screen_noamp_{tag}"]) < tol
    obl = O.obliquity_map(nX, nY, nT, dX, dY, dT, c0).astype(rdt)
    assert abs(O.beam_obliquity(u, obl) - G[f"oblscalar_{tag}"]) < 1e-5 * abs(G[f"oblscalar_{tag}"])


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("nT", [64, 65, 3, 801])
def test_fluxes(prec, nT):
    G = G32 if prec == "fp32" else G64
    N = 3.5 / (2 * 1540.0 ** 3 * 1000.0)
    col = G[f"col_{nT}"].reshape(1, 1, nT)
    for dZ, dTt in [(1.0e-4, 1.0e-8), (5.0e-4, 2.0e-8)]:
        t = f"{nT}_{dZ:g}_{dTt:g}"
        np.testing.assert_array_equal(O.flux_rusanov(col, N, dZ, dTt), G[f"rus_{t}"])
        np.testing.assert_array_equal(O.flux_rusanov_tvd(col, N, dZ, dTt, 1.7), G[f"tvd_{t}"])
        np.testing.assert_array_equal(O.flux_kt(col, N, dZ, dTt), G[f"kt_{t}"])
        np.testing.assert_array_equal(O.flux_kt(col, N, dZ, dTt, "minmod"), G[f"ktmm_{t}"])
        np.testing.assert_array_equal(O.flux_kt_adaptive(col, N, dZ, dTt, 0.05), G[f"ktad_{t}"])
        np.testing.assert_array_equal(O.flux_kt_percolumn(col, N, dZ, dTt, 0.05), G[f"ktad_{t}"])


def _solve(name, prec):
    u0, kw, ex = S.build_solve_inputs(name)
    p = O.OracleParams(**kw)
    for k, v in ex.items():
        setattr(p, k, v)
    return O.solve(u0, p, prec)


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
@pytest.mark.parametrize("name", list(S.SOLVE_SCENARIOS))
def test_solve_matches_reference(prec, name):
    G = G32 if prec == "fp32" else G64
    keys = ["field", "pnp", "ppp", "pI", "pIloss", "zaxis", "pax"]
    res = _solve(name, prec)
    for k, a in zip(keys, res):
        ref = G[f"solve_{name}_{k}"]
        assert a.shape == ref.shape, (k, a.shape, ref.shape)
        tol = 1e-12 if prec == "fp64" else 1e-6
        assert rel(a, ref) <= tol, (name, k, rel(a, ref))


def test_stability_violation_raises():
    u0, kw, _ = S.build_solve_inputs("strang_tvd_wendland")
    p = O.OracleParams(**kw)
    with pytest.raises(O.StabilityError):
        O.solve(u0 * 100.0, p, "fp32")


def test_march_runner_matches_solve():
    """The timing runner steps exactly like solve() (no screens/sources)."""
    for name in ["strang_kt_fw_sa", "lie_water_quadratic", "strang_tvd_wendland"]:
        u0, kw, ex = S.build_solve_inputs(name)
        p = O.OracleParams(**kw)
        ref = O.solve(u0, p, "fp32")
        m = O.OracleMarch(u0, p, "fp32").build()
        for _ in range(len(ref[5])):
            m.step()
        assert rel(m.u, ref[0]) < 1e-12
        assert rel(m.stats[1], ref[2][:, :, -1]) < 1e-6  # solve() stores float32
