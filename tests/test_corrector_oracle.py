"""The FP64 restatement of the corrector network: its analytic gradients agree
with central finite differences, and BF16 rounding is nearest-even."""
import numpy as np

import oracle.corrector as OC


def _params(seed):
    rng = np.random.default_rng(seed)
    P = {}
    for name, shp in [("W1", (64, 1, 5)), ("b1", (64,)), ("W2", (64, 64, 5)), ("b2", (64,)),
                      ("W3", (64, 64, 5)), ("b3", (64,)), ("W4", (1, 64, 5)), ("b4", (1,))]:
        fan = shp[1] * shp[2] if len(shp) == 3 else 1
        P[name] = rng.standard_normal(shp) * (np.sqrt(2.0 / fan) if len(shp) == 3 else 0.1)
    return P


def test_analytic_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    P = _params(1)
    x = rng.standard_normal((2, 20))
    tg = rng.standard_normal((2, 20)) * 0.3
    mk = np.ones((2, 20))
    mk[:, 0] = 0
    _, g = OC.loss_and_grads(x, tg, mk, P)
    h = 1e-6
    for name in OC.NAMES:
        flat = P[name].reshape(-1)
        for idx in rng.choice(flat.size, size=min(4, flat.size), replace=False):
            old = flat[idx]
            flat[idx] = old + h
            lp = OC.loss_only(x, tg, mk, P)
            flat[idx] = old - h
            lm = OC.loss_only(x, tg, mk, P)
            flat[idx] = old
            fd = (lp - lm) / (2 * h)
            an = g[name].reshape(-1)[idx]
            assert abs(fd - an) <= 1e-6 + 1e-5 * abs(fd), (name, idx, fd, an)


def test_padding_keeps_columns_apart():
    P = _params(2)
    x = np.random.default_rng(3).standard_normal((3, 16))
    y, _ = OC.forward(x, P)
    for b in range(3):
        yb, _ = OC.forward(x[b:b + 1], P)
        np.testing.assert_allclose(y[b], yb[0], rtol=0, atol=1e-12)


def test_bf16_rounding():
    a = np.array([1.0, 1.00390625, 1.005859375, -3.3e-5, 65504.0], np.float32)
    r = OC.bf16(a)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == np.float32(1.0078125)
    assert np.all(np.abs(r - a) <= np.abs(a) * 2.0 ** -8)
