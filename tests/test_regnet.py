"""The registration network's CPU oracle (oracle/regnet_oracle.py) checked on
the CPU: with its bf16 rounding switched off, its hand-written backward must
equal torch autograd of the same fp32 model.  This pins the oracle that the
GPU gradients are compared with (tests/test_regnet_gpu.py)."""
import numpy as np
import pytest

import regnet_oracle as ro


def _autograd(flat, x0, y, lam):
    torch = pytest.importorskip("torch")
    p = {k: torch.tensor(v, dtype=torch.float64, requires_grad=True) for k, v in ro.unflatten(flat).items()}
    x = torch.tensor(x0.reshape(-1, 3), dtype=torch.float64)
    B = y.shape[0]
    X1 = torch.relu(x @ p["w1"].T + p["b1"])
    X2 = torch.relu(X1 @ p["w2"].T + p["b2"])
    Y3 = torch.relu(X2 @ p["w3"].T + p["b3"])
    H0 = Y3.reshape(2 * B, ro.P, 256).max(dim=1).values.reshape(B, 512)
    H1 = torch.relu(H0 @ p["w4"].T + p["b4"])
    H2 = torch.relu(H1 @ p["w5"].T + p["b5"])
    out = H2 @ p["w6"].T + p["b6"]
    w = torch.tensor([lam] * 3 + [1.0] * 3, dtype=torch.float64)
    loss = (w * (out - torch.tensor(y, dtype=torch.float64)) ** 2).sum() / B
    loss.backward()
    return float(loss.detach()), np.concatenate([p[k].grad.numpy().reshape(-1) for k in ro.DIMS])


def test_oracle_backward_equals_autograd(monkeypatch):
    rng = np.random.default_rng(3)
    B = 4
    flat = np.concatenate([(rng.normal(0, 1 / np.sqrt(s[-1]), s) if len(s) == 2 else rng.normal(0, 0.1, s)).reshape(-1)
                           for s in ro.DIMS.values()]).astype(np.float32)
    x0 = rng.normal(0, 1, (B, 2, ro.P, 3)).astype(np.float32)
    y = rng.normal(0, 1, (B, 6)).astype(np.float32)
    monkeypatch.setattr(ro, "bf16", lambda a: np.asarray(a, np.float32))
    loss, g, _ = ro.loss_and_grad(flat, x0, y, 2.0)
    lref, gref = _autograd(flat, x0, y, 2.0)
    assert abs(loss - lref) <= 1e-4 * abs(lref)
    for k, (a, b) in _blocks(g, gref).items():
        assert np.linalg.norm(a - b) <= 1e-3 * np.linalg.norm(b) + 1e-6, k


def test_bf16_rounding_is_nearest_even():
    # 1 + 2^-8 is halfway between 1 and 1 + 2^-7: ties go to the even mantissa (1);
    # 1 + 3 * 2^-8 is halfway between 1 + 2^-7 and 1 + 2^-6: ties go to 1 + 2^-6
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 1.0 + 2 ** -7], np.float32)
    want = np.array([1.0, 1.0, 1.0 + 2 ** -6, -2.5, 1.0 + 2 ** -7], np.float32)
    assert np.array_equal(ro.bf16(x), want)


def _blocks(a, b):
    out, o = {}, 0
    for k, s in ro.DIMS.items():
        n = int(np.prod(s))
        out[k] = (a[o:o + n], b[o:o + n])
        o += n
    return out
