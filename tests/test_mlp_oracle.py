"""The NumPy restatement of the surrogate MLP (oracle/mlp_ref.py), pinned
on the CPU: its BF16 rounding against torch's float32 -> bfloat16
conversion, and its hand-written backward pass against centred finite
differences of the same network in FP64."""
import mlp_ref
import numpy as np
import torch


def _layout(n_in, n_hid, nh, n_out):
    out, off = [], 0
    for l in range(nh + 1):
        din = n_in if l == 0 else n_hid
        dout = n_out if l == nh else n_hid
        out.append((off, off + din * dout, dout, din))
        off += din * dout + dout
    return out, off


def test_bf16_rounding_matches_torch():
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.standard_normal(100000) * 10.0 ** rng.integers(-30, 30, 100000),
                        np.array([0.0, -0.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 65504.0, 3.0e38])]).astype(np.float32)
    ref = torch.as_tensor(x).to(torch.bfloat16).float().numpy().astype(np.float64)
    np.testing.assert_array_equal(mlp_ref.bf16(x), ref)


def test_backward_matches_finite_differences():
    layout, n = _layout(6, 12, 2, 4)
    rng = np.random.default_rng(1)
    p = rng.standard_normal(n) * 0.4
    x = rng.standard_normal((50, 6))
    t = np.zeros((50, 16))
    t[:, 0:4:2] = rng.uniform(size=(50, 2)) < 0.5
    t[:, 1:4:2] = rng.standard_normal((50, 2))
    _, g = mlp_ref.loss_grad(p, layout, x, t, quant=False)
    d = rng.standard_normal(n)
    h = 1e-6
    lp, _ = mlp_ref.loss_grad(p + h * d, layout, x, t, quant=False)
    lm, _ = mlp_ref.loss_grad(p - h * d, layout, x, t, quant=False)
    fd = (lp - lm) / (2 * h)
    assert abs(fd - g @ d) <= 1e-7 * max(abs(fd), 1.0), (fd, g @ d)
