"""The learned surrogate of the ICE4_SLOW rates on the GPU.

* the sampling kernel (features, plain-kernel slow rates as targets) against
  the host build of the same code;
* with an empty training envelope every point takes the plain path: the
  surrogate-assisted rain_ice and chained step equal the plain ones bit for
  bit (the in-launch fall-back);
* training on the device kernels lowers the held-out error of every rate;
* the trained network shipped with the package (ice3gb/data/
  slow_surrogate.npz): per-rate held-out error, and the surrogate-assisted
  step against the plain FP64 step, per field, compared with the same step
  without the network (all learned rates zero) — what the network gains."""
import ctypes
import os

import numpy as np
import pytest
import torch

from test_rain_ice_host import host_lib  # noqa: F401  (host build of the sampling, a fixture)

pytestmark = pytest.mark.gpu

DT = 50.0
NK = 90
INOUT = ("ths", "rvs", "rcs", "rrs", "ris", "rss", "rgs", "ci_t")


def _chained(nij, seed):
    from ice3gb.state import make_state
    from ice3gb.surrogate import chained_rain_ice_state
    st = make_state(nij, NK, seed=seed, precip=True, device="cuda")
    return chained_rain_ice_state(st, DT)


def _empty_envelope():
    return {"mean": np.zeros(16, np.float32), "inv_std": np.ones(16, np.float32),
            "lo": np.ones(16, np.float32), "hi": -np.ones(16, np.float32)}


def test_sample_matches_host_build(host_lib):  # noqa: F811
    from ice3gb.components import RainIce
    from ice3gb.surrogate import sample
    ri = RainIce(table="phyex")
    state = _chained(32 * 32, seed=3)
    smp = sample(ri, state, DT, targets=True)
    c = ri.prepare({k: (v.cpu().numpy() if isinstance(v, torch.Tensor) else v) for k, v in state.items()})
    n = c["nij"] * c["nk"]
    feat = np.zeros((n, 16), dtype=np.float32)
    rate = np.zeros((n, 5))
    micro = np.zeros(n, dtype=np.uint8)
    host_lib.sur_sample_host.restype = ctypes.c_long
    cnt = host_lib.sur_sample_host(ctypes.byref(ri.table.consts), ctypes.byref(ri.table.luts), c["nij"], c["nk"],
                                   ctypes.c_double(DT), ctypes.byref(c["f"]), feat.ctypes.data_as(ctypes.c_void_p),
                                   rate.ctypes.data_as(ctypes.c_void_p), micro.ctypes.data_as(ctypes.c_void_p))
    rows = smp["point_of_row"].cpu().numpy()
    assert cnt == len(rows) == smp["stats"]["micro"] > 0
    np.testing.assert_array_equal(rows, np.nonzero(micro)[0])
    fd = smp["features"].cpu().numpy().astype(np.float64)
    fh = feat[rows].astype(np.float64)
    # FP32 features: the host's and the device's logf / expf may differ in the last bits
    assert np.all(np.abs(fd - fh) <= 1e-5 * (np.abs(fh) + 1.0))
    td = smp["targets"].cpu().numpy().astype(np.float64)
    rh = rate[rows]
    np.testing.assert_array_equal(td[:, 0:10:2], (rh != 0).astype(np.float64))
    rf = rh.astype(np.float32).astype(np.float64)
    assert np.all(np.abs(td[:, 10:15] - rf) <= 4e-7 * np.abs(rf) + 1e-38)


def test_inference_features_equal_training_features():
    """The feature-only sampling (inference) and the sampling with targets
    (training) give the same features bit for bit."""
    from ice3gb.components import RainIce
    from ice3gb.surrogate import sample
    ri = RainIce(table="phyex")
    state = _chained(96 * 96, seed=8)
    a = sample(ri, state, DT, targets=True)
    b = sample(ri, state, DT, targets=False)
    assert torch.equal(a["point_of_row"], b["point_of_row"])
    assert torch.equal(a["features"], b["features"])


def test_empty_envelope_is_the_plain_path():
    from ice3gb.components import RainIce
    from ice3gb.surrogate import SlowSurrogate
    ri = RainIce(table="phyex")
    state = _chained(64 * 64, seed=4)
    plain, dp = ri(state, DT)
    sur = SlowSurrogate(norm=_empty_envelope(), seed=3)
    got, dg = ri(state, DT, surrogate=sur)
    st = ri.surrogate_stats
    assert st["micro"] > 0 and st["outside_envelope"] == st["micro"] and st["used"] == 0
    for k in INOUT:
        assert torch.equal(got[k], plain[k]), k
    for k in dp:
        assert torch.equal(dg[k], dp[k]), k


def test_physics_step_surrogate_empty_envelope_is_plain():
    from ice3gb import _abi
    from ice3gb.components import Ice3Handle
    from ice3gb.constants import build_table
    from ice3gb.state import make_state
    from ice3gb.surrogate import SlowSurrogate, physics_step_surrogate
    import bench
    nij = 48 * 48
    st = bench.step_state(make_state(nij, NK, seed=9, precip=True, device="cuda"))
    h = Ice3Handle(build_table(table="phyex"))
    res = []
    for use_sur in (False, True):
        work = {k: st[k].clone() for k in bench.STEP_INOUT}
        outs = {k: torch.empty((NK, nij), dtype=torch.float64, device="cuda") for k in bench.STEP_OUT3}
        outs.update({k: torch.empty((nij,), dtype=torch.float64, device="cuda") for k in bench.STEP_OUT2})
        f = _abi.StepFields()
        for k in bench.STEP_IN + ("sea", "town"):
            setattr(f, k, ctypes.c_void_p(st[k].data_ptr()))
        for k, v in {**work, **outs}.items():
            setattr(f, k, ctypes.c_void_p(v.data_ptr()))
        opt = _abi.RainIceOptions(-1, -1, -1, 0, 0)
        if use_sur:
            stats = physics_step_surrogate(h, SlowSurrogate(norm=_empty_envelope()), f, nij, NK, DT, opt)
            assert stats["used"] == 0 and stats["outside_envelope"] == stats["micro"] > 0
        else:
            _abi.check(h.lib.ice3gb_physics_step(h.h, nij, NK, DT, ctypes.byref(opt), ctypes.byref(f),
                                                 ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)),
                       h.h, "ice3gb_physics_step")
        torch.cuda.synchronize()
        res.append({**work, **outs})
    for k in res[0]:
        assert torch.equal(res[0][k], res[1][k]), k


def test_training_lowers_every_rate_error():
    from ice3gb.surrogate import RATES, SlowSurrogate, training_set
    raw, tgt = training_set(1 << 18, nij=4096, seed=5000)
    ev_raw, ev_tgt = training_set(1 << 16, nij=4096, seed=6000)
    sur = SlowSurrogate(seed=1)
    sur.norm = sur.fit_norm(raw)
    e0 = sur.rate_errors(ev_raw, ev_tgt)
    sur.train(raw, tgt, epochs=4, batch=4096, lr=2e-3, warmup=50)
    e1 = sur.rate_errors(ev_raw, ev_tgt)
    for r in RATES:
        if e1[r].get("points", 0) < 100:          # too rare in this sample to measure
            continue
        assert e1[r]["nrmse"] < 0.5 * e0[r]["nrmse"], (r, e0[r], e1[r])
        assert e1[r]["activity_acc"] > 0.9, (r, e1[r])


TRAINED = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "dwarf-p-ice3_gb300", "ice3gb", "data",
                       "slow_surrogate.npz")


@pytest.mark.skipif(not os.path.exists(TRAINED), reason="no trained surrogate shipped")
def test_trained_surrogate_gain_over_no_network():
    """Per field, the surrogate-assisted rain_ice stays closer to the plain
    FP64 step than the same step without the network (learned rates all
    zero, same envelope and fix-up): the network's gain."""
    from ice3gb.components import RainIce
    from ice3gb.surrogate import SlowSurrogate
    sur = SlowSurrogate.load(TRAINED)
    silent = SlowSurrogate.silent(sur.norm)
    ri = RainIce(table="phyex")
    state = _chained(128 * 128, seed=424242)                # a seed outside the training set
    plain, _ = ri(state, DT)
    with_net, _ = ri(state, DT, surrogate=sur)
    st = dict(ri.surrogate_stats)
    without, _ = ri(state, DT, surrogate=silent)
    assert st["used"] >= 0.9 * st["micro"], st
    assert st["fixup_fallback"] <= 0.01 * st["micro"], st
    gains = {}
    for k in ("ths", "rvs", "ris", "rss", "rgs"):
        d = state[k]                                        # the step's change of the source
        scale = float(torch.sqrt(((plain[k] - d) ** 2).mean()))
        e_with = float(torch.sqrt(((with_net[k] - plain[k]) ** 2).mean())) / scale
        e_without = float(torch.sqrt(((without[k] - plain[k]) ** 2).mean())) / scale
        gains[k] = (e_with, e_without)
        assert e_with <= 0.25 * e_without, (k, e_with, e_without)
    print(gains)
