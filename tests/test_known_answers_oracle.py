"""The oracle against the reference's published known answers (CPU).

The cheap cases run live (DC invariance, isolated Burgers-step order,
attenuation and Kramers-Kronig dispersion); the heavier ones (boundary
reflection, march convergence, pistons) were run once by
tests/golden/make_known_answers.py and their stored metrics are held to the
published figures here, so the fixture the GPU tests compare against is
itself pinned."""
import json
import os

import numpy as np
import pytest

import known_answers as K
import oracle.asm_oracle as O

with open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")) as _f:
    FIX = json.load(_f)


def _solve(u0, kw, prec="fp32"):
    return O.solve(u0, O.OracleParams(**kw), prec)


def test_dc_invariance():
    peaks = []
    for nT in (120, 240, 480):
        u0, kw = K.dc_case(nT)
        peak, growth = K.dc_metrics(u0, _solve(u0, kw, "fp64")[0])
        assert growth <= 1.0
        peaks.append(peak)
    assert (max(peaks) - min(peaks)) / min(peaks) <= 0.05


@pytest.mark.parametrize("name,fn,lo,hi", [("rusanov", O.flux_rusanov, 0.95, 1.15),
                                           ("kt", O.flux_kt, 1.75, 2.1)])
def test_isolated_burgers_step_order(name, fn, lo, hi):
    u0, dT, N = K.order_column()

    def run(dz):
        u = u0.reshape(1, 1, -1)
        for _ in range(int(round(K.ORDER_Z / dz))):
            u = np.asarray(fn(u, N, dz, dT))
        return u[0, 0]

    ref = run(K.ORDER_REF_DZ).astype(np.float64)
    rate, _ = K.order_rate([run(d) for d in K.ORDER_DZ], ref)
    assert lo <= rate <= hi, rate
    assert abs(rate - K.PUBLISHED["order"][name]) <= 0.1


def test_attenuation_and_kk():
    u0, kw = K.attenuation_case()
    r = _solve(u0, kw)
    a_rms, c_rms = K.attenuation_metrics(u0, r[0], r[5], kw)
    assert a_rms < 1e-3 and c_rms < 0.05, (a_rms, c_rms)


def test_stored_metrics_match_published_figures():
    for name, pub in K.PUBLISHED["reflection"].items():
        assert abs(FIX["reflection"][name] - pub) <= 0.01 * pub + 5e-5, name
    kt = FIX["convergence"]["split_kt"]["pair_errors"]
    assert abs(kt[0] - 8.3e-4) <= 0.05 * 8.3e-4 and abs(kt[1] - 2.2e-4) <= 0.05 * 2.2e-4
    assert 1.9 <= FIX["convergence"]["split_kt"]["rate"] <= 2.2
    for n in ("sequential", "split_rusanov"):
        assert 0.9 <= FIX["convergence"][n]["rate"] <= 1.2
    assert abs(FIX["baffled"]["onaxis_rms"] - K.PUBLISHED["baffled_onaxis_rms"]) <= 5e-4
    assert abs(FIX["focused"]["onaxis_rms"] - K.PUBLISHED["focused_onaxis_rms"]) <= 5e-4
    assert abs(FIX["focused"]["lateral_rms"] - K.PUBLISHED["focused_lateral_rms"]) <= 1e-4


def test_riemann_shock():
    """The KT step against the exact shock (below the published errors of the
    reference's first-order finite-volume KT); the standard Rusanov step of
    the reference carries twice the flux, so its shock runs at speed 2."""
    _, dT, _ = K.riemann_column()
    kt = K.riemann_errors(lambda u, dz: np.asarray(O.flux_kt(u.reshape(1, 1, -1), 1.0, dz, dT))[0, 0])
    assert all(e < p for e, p in zip(kt, K.RIEMANN_PUBLISHED_KT)), kt
    ru = K.riemann_errors(
        lambda u, dz: np.asarray(O.flux_rusanov(u.reshape(1, 1, -1), 1.0, dz, dT))[0, 0], speed=2.0)
    assert max(ru) < 0.045, ru
