"""Learned corrector kernels against the FP64 CPU restatement of the network:
forward, loss and every parameter gradient; a short training run lowers the
loss."""
import numpy as np
import pytest

import oracle.corrector as OC

pytestmark = pytest.mark.gpu


def _batch(ncols, nT, seed):
    rng = np.random.default_rng(seed)
    t = np.linspace(0, 1, nT)
    x = np.stack([np.sin(2 * np.pi * rng.uniform(2, 9) * t + rng.uniform(0, 6))
                  * np.exp(-((t - rng.uniform(0.3, 0.7)) / 0.2) ** 2) for _ in range(ncols)])
    x = (x + 0.05 * rng.standard_normal(x.shape)).astype(np.float32)
    target = (0.1 * np.roll(x, 1, axis=1) - 0.05 * x ** 2).astype(np.float32)
    mask = np.ones_like(x)
    mask[:, 0] = mask[:, -1] = 0.0
    return x, target, mask


def _rel(a, b):
    return float(np.linalg.norm(np.ravel(a) - np.ravel(b)) / (np.linalg.norm(np.ravel(b)) + 1e-30))


def _oracle_params(theta, bf16_gemm):
    from angularspectrum_heterogeneous_gb300 import corrector as CR
    P = {k: v.astype(np.float64) for k, v in CR.to_dict(theta).items()}
    if bf16_gemm:  # the GPU runs the 64x64 layers with BF16 weights
        for k in ("W2", "W3"):
            P[k] = OC.bf16(P[k]).astype(np.float64)
    return P


def test_forward_matches_oracle():
    import torch
    from angularspectrum_heterogeneous_gb300 import corrector as CR
    theta = CR.init_params(3, last_scale=1.0)
    net = CR.Corrector(theta)
    try:
        x, _, _ = _batch(6, 128, 1)
        y = net.forward(torch.from_numpy(x).cuda()).cpu().numpy()
        yr, _ = OC.forward(x, _oracle_params(theta, True))
        # BF16 weights emulated in the oracle; activations are BF16 on the GPU
        assert _rel(y, yr) < 2e-2, _rel(y, yr)
        y64, _ = OC.forward(x, _oracle_params(theta, False))
        assert _rel(y, y64) < 3e-2
    finally:
        net.close()


def test_gradients_match_oracle():
    import torch
    from angularspectrum_heterogeneous_gb300 import corrector as CR
    theta = CR.init_params(5, last_scale=1.0)
    net = CR.Corrector(theta)
    try:
        x, tg, mk = _batch(4, 256, 2)
        d = [torch.from_numpy(a).cuda() for a in (x, tg, mk)]
        loss, g = net.train_step(*d, lr=0.0, want_grad=True)
        lr_, gr = OC.loss_and_grads(x, tg, mk, _oracle_params(theta, True))
        assert abs(loss - lr_) / lr_ < 2e-2, (loss, lr_)
        gd = CR.to_dict(g)
        for name, _ in CR.SHAPES:
            a, b = gd[name].ravel(), gr[name].ravel()
            cos = float(a @ b / (np.linalg.norm(a) * np.linalg.norm(b) + 1e-30))
            assert cos > 0.995 and _rel(a, b) < 8e-2, (name, cos, _rel(a, b))
        # no update with lr = 0
        assert np.array_equal(net.get_params(), theta)
    finally:
        net.close()


def test_training_lowers_the_loss():
    import torch
    from angularspectrum_heterogeneous_gb300 import corrector as CR
    net = CR.Corrector(CR.init_params(7))
    try:
        x, tg, mk = _batch(32, 256, 3)
        d = [torch.from_numpy(a).cuda() for a in (x, tg, mk)]
        first = net.train_step(*d, lr=0.0)
        for _ in range(60):
            last = net.train_step(*d, lr=2e-3)
        assert last < 0.3 * first, (first, last)
    finally:
        net.close()
