"""Host-side logic of the slow-rate surrogate (no GPU): the target coding
and its decoding as the kernel decodes it, and the feature normalisation /
training envelope."""
import numpy as np
import torch

from ice3gb import surrogate as S


def test_decode_inverts_encode():
    rng = np.random.default_rng(0)
    r = rng.standard_normal((5000, 5)) * 10.0 ** rng.uniform(-16, 2, (5000, 5))
    r[rng.uniform(size=r.shape) < 0.3] = 0.0
    r[:, [0, 2, 3]] = np.abs(r[:, [0, 2, 3]])
    t = S.encode(torch.as_tensor(r))
    y = torch.zeros((5000, 10))
    y[:, 0::2] = torch.where(t[:, 0:10:2] > 0.5, 1.0, -1.0)
    y[:, 1::2] = t[:, 1:10:2]
    back = S.decode(y).double().numpy()
    # FP32 coding: relative error of a few float ulps times SUR_AMP * |coded value|
    assert np.all(np.abs(back - r) <= 2e-5 * np.abs(r) + 1e-30)
    np.testing.assert_array_equal(back == 0, r == 0)


def test_decode_clips_the_coded_value():
    y = torch.tensor([[1.0, 9.0] * 5, [1.0, -9.0] * 5, [-1.0, 3.0] * 5])
    r = S.decode(y)
    big = float(np.float32(1e-12) * np.sinh(np.float32(40.0)))
    assert torch.allclose(r[0], torch.full((5,), big)) and torch.allclose(r[1], torch.full((5,), -big))
    assert torch.all(r[2] == 0)


def test_norm_envelope_contains_training_features():
    g = torch.Generator().manual_seed(1)
    raw = torch.randn((20000, 16), generator=g, dtype=torch.float64) * torch.linspace(0.1, 50, 16) + 7.0
    raw[:, 11] = 50.0                                   # a constant feature (dt)
    norm = S.SlowSurrogate.fit_norm(raw)
    z = (raw.float() - torch.as_tensor(norm["mean"])) * torch.as_tensor(norm["inv_std"])
    assert bool(((z >= torch.as_tensor(norm["lo"])) & (z <= torch.as_tensor(norm["hi"]))).all())
    assert abs(float(z[:, 0].std()) - 1.0) < 1e-3 and float(z[:, 11].abs().max()) == 0.0
    out = z.clone()
    out[:, 11] = 1.0                                    # another dt leaves the envelope
    assert not bool((out[:, 11] <= float(norm["hi"][11])).any())
