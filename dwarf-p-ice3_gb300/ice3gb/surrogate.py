"""Learned surrogate of the ICE4_SLOW rates inside rain_ice.

The five slow processes of PHYEX ICE4 (mode_ice4_slow.F90: RCHONI
homogeneous freezing of cloud droplets, RVDEPS deposition on snow, RIAGGS
aggregation of ice on snow, RIAUTS ice autoconversion, RVDEPG deposition on
graupel), which the reference reaches from ``RainIceJAX``
(src/ice3/jax/rain_ice.py:181), are replaced at the first hard pass of each
micro point by a per-point MLP (16 features -> 3 x 256 GELU -> 10 outputs,
BF16 weights, FP32 accumulation on the tcgen05 tensor cores; ice3gb.mlp).

* Features and targets come from the plain kernel itself
  (``ice3gb_surrogate_sample``): 16 FP32 features of a micro point's state
  at the start of the step and the five rates the plain FP64 code computes
  at its first hard pass.
* Training runs on the GPU through the library's own forward and backward
  kernels (``Mlp.train_step``, Adam).
* Inference (``RainIce(..., surrogate=...)``, ``physics_step_surrogate``)
  samples the features, runs the network, then the rain_ice kernel takes the
  learned rates where the point lies inside the training envelope and passes
  the fix-up check, and runs the plain path elsewhere, in the same launch.
  Each process keeps its exact activity condition and the sign / cap of its
  rate; the network gives the magnitude (and a "nonzero" logit).

Output coding per rate k: y[2k] = logit of "rate != 0", y[2k+1] =
asinh(rate / 1e-12) / 10, decoded as 1e-12 sinh(10 clip(y, -4, 4)) where
the logit is positive.
"""
from __future__ import annotations

import ctypes
import math
import os
from typing import Dict, List, Mapping, Optional, Tuple

import numpy as np
import torch

from . import _abi
from .mlp import Mlp

RATES = ("rchoni", "rvdeps", "riaggs", "riauts", "rvdepg")
FEATURES = ("T", "ln_p", "ln_rho", "ln_rv", "ln_rc", "ln_rr", "ln_ri", "ln_rs", "ln_rg", "cldfr", "exn", "dt",
            "ln_lbda_r", "ln_lbda_s", "ln_lbda_g", "ssi")
SCALE, AMP, CLIP = 1e-12, 10.0, 4.0
DEFAULT_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "slow_surrogate.npz")


def _ptr(t: Optional[torch.Tensor]) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr() if t is not None else 0)


def _stream() -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def encode(rates: torch.Tensor) -> torch.Tensor:
    """[n, 5] rates -> [n, 16] target rows as the sampling kernel writes them."""
    n = rates.shape[0]
    t = torch.zeros((n, 16), dtype=torch.float32, device=rates.device)
    r = rates.double()
    t[:, 0:10:2] = (r != 0).float()
    t[:, 1:10:2] = (torch.asinh(r / SCALE) / AMP).float()
    t[:, 10:15] = r.float()
    return t


def decode(y: torch.Tensor) -> torch.Tensor:
    """[n, 10] network outputs -> [n, 5] rates (FP32 arithmetic, as the kernel)."""
    u = y[:, 1:10:2].float().clamp(-CLIP, CLIP)
    r = np.float32(SCALE) * torch.sinh(np.float32(AMP) * u)
    return torch.where(y[:, 0:10:2] > 0, r, torch.zeros_like(r))


# ---------------------------------------------------------------------------- sampling

def sample(rain_ice, state: Mapping, dt: float, norm: Optional["_abi.SurrogateNorm"] = None,
           targets: bool = True, cap: Optional[int] = None) -> Dict:
    """Features (and targets) of the micro points of one rain_ice call on
    ``state`` (RainIce state keys, CUDA tensors), rows sorted by grid point.

    Returns {"features" [rows, 16], "targets" [rows, 16] or None,
    "point_of_row" [rows] int64, "stats" {counter: value}}."""
    c = rain_ice.prepare(state)
    nij, nk = c["nij"], c["nk"]
    n = nij * nk
    cap = n if cap is None else int(cap)
    dev = c["fields"]["tht"].device
    feat = torch.empty((max(cap, 1), 16), dtype=torch.float32, device=dev)
    tgt = torch.empty((max(cap, 1), 16), dtype=torch.float32, device=dev) if targets else None
    por = torch.empty(max(cap, 1), dtype=torch.int64, device=dev)
    ctr = torch.zeros(1 + _abi.SUR_NSTATS, dtype=torch.int64, device=dev)
    h = rain_ice.handle
    normp = ctypes.byref(norm) if norm is not None else None
    _abi.check(h.lib.ice3gb_surrogate_sample(h.h, nij, nk, float(dt), ctypes.byref(c["f"]), normp, cap, _ptr(feat),
                                             _ptr(tgt), _ptr(por), None, _ptr(ctr), _stream()), h.h,
               "ice3gb_surrogate_sample")
    counters = ctr.cpu().numpy()
    rows = int(min(counters[0], cap))
    por = por[:rows]
    order = torch.argsort(por)
    out = {"features": feat[:rows][order], "targets": tgt[:rows][order] if targets else None,
           "point_of_row": por[order], "stats": dict(zip(_abi.SUR_STATS, (int(v) for v in counters[1:])))}
    return out


def chained_rain_ice_state(st: Mapping[str, torch.Tensor], dt: float, table: str = "phyex") -> Dict:
    """The RainIce state that rain_ice sees inside the chained step
    (ice_adjust -> rain_ice -> ice_adjust) for a make_state(precip=True)
    dict: the time-t state, cloud fraction and subgrid partition from the
    first adjustment, the sources after it."""
    from .components import IA_INOUT, IA_OUTPUTS, IceAdjust
    from .state import rain_ice_state
    ia = IceAdjust(table=table)
    names = ("sigqsat", "pabs", "sigs", "th", "exn", "exn_ref", "rho_dry_ref", "rv", "rc", "ri", "rr", "rs", "rg",
             "cf_mf", "rc_mf", "ri_mf", "rvs", "rcs", "ris", "ths")
    outs = dict(zip(IA_OUTPUTS + IA_INOUT, ia(**{k: st[k] for k in names}, timestep=dt)))
    ri = dict(rain_ice_state(st))
    for k in ("cldfr", "hlc_hrc", "hlc_hcf", "hli_hri", "hli_hcf", "ths", "rvs", "rcs", "ris"):
        ri[k] = outs[k]
    return ri


def training_set(n_points: int, nij: int = 65536, nk: int = 90, seed: int = 1000, dt: float = 50.0,
                 table: str = "phyex", chained: bool = True) -> Tuple[torch.Tensor, torch.Tensor]:
    """(raw features [n, 16], targets [n, 16]) of ``n_points`` micro points
    from seeded synthetic AROME-like states (ice3gb.state.make_state with
    precipitation), through the plain kernel's own sampling."""
    from .components import RainIce
    from .state import make_state, rain_ice_state
    ri = RainIce(table=table)
    feats, tgts, have, s = [], [], 0, seed
    dev = torch.device("cuda", torch.cuda.current_device())
    while have < n_points:
        st = make_state(nij, nk, seed=s, precip=True, device=dev, dt=dt)
        state = chained_rain_ice_state(st, dt, table) if chained else rain_ice_state(st)
        smp = sample(ri, state, dt, targets=True)
        take = min(n_points - have, smp["features"].shape[0])
        feats.append(smp["features"][:take].clone())
        tgts.append(smp["targets"][:take].clone())
        have += take
        s += 1
        del st, state, smp
    return torch.cat(feats), torch.cat(tgts)


# ---------------------------------------------------------------------------- the surrogate

class SlowSurrogate:
    """The network and its feature normalisation / envelope."""

    def __init__(self, mlp: Optional[Mlp] = None, norm: Optional[Dict[str, np.ndarray]] = None, seed: int = 0,
                 n_hidden: int = 256, n_hidden_layers: int = 3):
        self.mlp = mlp if mlp is not None else Mlp(16, n_hidden, n_hidden_layers, 10, seed=seed)
        self.norm = norm
        self.history: List[Dict] = []

    # ---- normalisation ------------------------------------------------------
    @staticmethod
    def fit_norm(raw: torch.Tensor, margin: float = 0.05) -> Dict[str, np.ndarray]:
        """Mean / spread of the raw features and the envelope of the
        standardised training features widened by ``margin`` of its range."""
        x = raw.double()
        mean = x.mean(dim=0)
        std = x.std(dim=0)
        inv = torch.where(std > 0, 1.0 / std.clamp_min(1e-300), torch.ones_like(std))
        z = (x - mean) * inv
        lo, hi = z.min(dim=0).values, z.max(dim=0).values
        w = (hi - lo).clamp_min(1e-6)
        f = lambda t: t.cpu().numpy().astype(np.float32)  # noqa: E731
        return {"mean": f(mean), "inv_std": f(inv), "lo": f(lo - margin * w), "hi": f(hi + margin * w)}

    def norm_struct(self) -> _abi.SurrogateNorm:
        if self.norm is None:
            raise RuntimeError("the surrogate has no normalisation (train or load it first)")
        s = _abi.SurrogateNorm()
        for k in ("mean", "inv_std", "lo", "hi"):
            getattr(s, k)[:] = [float(v) for v in self.norm[k]]
        return s

    def standardize(self, raw: torch.Tensor) -> torch.Tensor:
        m = torch.as_tensor(self.norm["mean"], device=raw.device)
        i = torch.as_tensor(self.norm["inv_std"], device=raw.device)
        return ((raw - m) * i).float().contiguous()

    def inside(self, z: torch.Tensor) -> torch.Tensor:
        lo = torch.as_tensor(self.norm["lo"], device=z.device)
        hi = torch.as_tensor(self.norm["hi"], device=z.device)
        return ((z >= lo) & (z <= hi)).all(dim=1)

    # ---- training -------------------------------------------------------------
    def train(self, raw: torch.Tensor, targets: torch.Tensor, epochs: int = 10, batch: int = 16384,
              lr: float = 2e-3, lr_min: float = 2e-5, warmup: int = 200, seed: int = 0,
              log_every: int = 0) -> List[Dict]:
        """Adam with linear warm-up and cosine decay on the device kernels.
        Fits the normalisation first if there is none."""
        if self.norm is None:
            self.norm = self.fit_norm(raw)
        x = self.standardize(raw)
        t = targets.float().contiguous()
        n = x.shape[0]
        steps_per_epoch = max(n // batch, 1)
        total = epochs * steps_per_epoch
        gen = torch.Generator(device=x.device)
        gen.manual_seed(seed)
        lbuf = torch.zeros(1, dtype=torch.float32, device=x.device)
        acc = torch.zeros(1, dtype=torch.float32, device=x.device)
        step = 0
        for ep in range(epochs):
            perm = torch.randperm(n, generator=gen, device=x.device)
            acc.zero_()
            for b in range(steps_per_epoch):
                idx = perm[b * batch:(b + 1) * batch]
                if step < warmup:
                    a = lr * (step + 1) / warmup
                else:
                    q = (step - warmup) / max(total - warmup, 1)
                    a = lr_min + 0.5 * (lr - lr_min) * (1.0 + math.cos(math.pi * q))
                self.mlp.train_step(x[idx], t[idx], a, lbuf)
                acc += lbuf
                step += 1
                if log_every and step % log_every == 0:
                    print(f"step {step}/{total} lr {a:.2e} loss {float(lbuf.item()):.5f}", flush=True)
            rec = {"epoch": ep, "mean_loss": float(acc.item()) / steps_per_epoch}
            self.history.append(rec)
        self.mlp.check()
        return self.history

    # ---- inference / evaluation -------------------------------------------------
    def predict(self, raw: torch.Tensor) -> torch.Tensor:
        """Rates [n, 5] (FP32, decoded as the kernel decodes them)."""
        return decode(self.mlp(self.standardize(raw)))

    def rate_errors(self, raw: torch.Tensor, targets: torch.Tensor) -> Dict[str, Dict[str, float]]:
        """Per slow rate: RMSE (kg/kg/s) over the points where the plain rate
        or the prediction is nonzero, RMS of the plain rate where it is
        nonzero ("points"), their ratio, the median relative error there, and
        the share of all points whose nonzero/zero status is predicted right."""
        pred = self.predict(raw).double()
        ref = targets[:, 10:15].double()
        out = {}
        for k, name in enumerate(RATES):
            p, r = pred[:, k], ref[:, k]
            nz = r != 0
            m = nz | (p != 0)
            if int(nz.sum()) == 0:
                out[name] = {"points": 0, "predicted_nonzero": int(m.sum())}
                continue
            d = (p - r)[m]
            rmse = float(torch.sqrt((d * d).mean()))
            rms = float(torch.sqrt((r[nz] * r[nz]).mean()))
            rel = ((p - r).abs() / r.abs())[nz]
            out[name] = {"points": int(nz.sum()), "rmse": rmse, "rms": rms, "nrmse": rmse / rms,
                         "median_rel_err": float(rel.median()),
                         "activity_acc": float(((p != 0) == nz).double().mean())}
        return out

    # ---- persistence --------------------------------------------------------------
    def save(self, path: str = DEFAULT_PATH) -> None:
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        n_in, n_hid, nh, n_out = self.mlp.shape
        np.savez(path, params=self.mlp.get_params(), shape=np.array([n_in, n_hid, nh, n_out], dtype=np.int32),
                 **{f"norm_{k}": v for k, v in self.norm.items()})

    @classmethod
    def load(cls, path: str = DEFAULT_PATH) -> "SlowSurrogate":
        d = np.load(path)
        n_in, n_hid, nh, n_out = (int(v) for v in d["shape"])
        mlp = Mlp(n_in, n_hid, nh, n_out, seed=0)
        mlp.set_params(d["params"])
        norm = {k: d[f"norm_{k}"].astype(np.float32) for k in ("mean", "inv_std", "lo", "hi")}
        return cls(mlp, norm)

    @classmethod
    def silent(cls, norm: Dict[str, np.ndarray], n_hidden: int = 256, n_hidden_layers: int = 3) -> "SlowSurrogate":
        """The method without the network: a surrogate whose logits are all
        negative (every learned slow rate zero), same envelope."""
        s = cls(None, norm, n_hidden=n_hidden, n_hidden_layers=n_hidden_layers)
        p = s.mlp.get_params()
        wo, bo, o, i = s.mlp.layout()[-1]
        p[wo:wo + o * i] = 0.0
        p[bo:bo + o] = 0.0
        p[bo:bo + o:2] = -10.0
        s.mlp.set_params(p)
        return s


# ---------------------------------------------------------------------------- chained step

def physics_step_surrogate(handle, surrogate: SlowSurrogate, fields: "_abi.StepFields", nij: int, nk: int,
                           dt: float, opt: Optional["_abi.RainIceOptions"] = None) -> Dict[str, int]:
    """ice3gb_physics_step_surrogate on an already filled StepFields (device
    pointers); returns the surrogate counters of the step."""
    opt = opt if opt is not None else _abi.RainIceOptions(-1, -1, -1, 0, 0)
    stats = (ctypes.c_uint64 * _abi.SUR_NSTATS)()
    norm = surrogate.norm_struct()
    _abi.check(handle.lib.ice3gb_physics_step_surrogate(handle.h, surrogate.mlp.h, nij, nk, float(dt),
                                                        ctypes.byref(opt), ctypes.byref(fields), ctypes.byref(norm),
                                                        stats, _stream()), handle.h, "ice3gb_physics_step_surrogate")
    return dict(zip(_abi.SUR_STATS, (int(v) for v in stats)))


def time_inference(sur: SlowSurrogate, rows: int, reps: int = 5) -> Dict[str, float]:
    """Device time of the network on `rows` standardised feature rows (CUDA
    events on the current stream, after one warm-up call): ms per call and
    the tensor throughput it implies (2 * multiply-adds of the layers)."""
    n_in, n_hid, nh, n_out = sur.mlp.shape
    gen = torch.Generator(device="cuda")
    gen.manual_seed(0)
    x = torch.randn((rows, n_in), generator=gen, device="cuda", dtype=torch.float32)
    sur.mlp(x)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        sur.mlp(x)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    flop = 2.0 * rows * (n_in * n_hid + (nh - 1) * n_hid * n_hid + n_hid * n_out)
    return {"rows": rows, "ms": ms, "tflops": flop / (ms * 1e-3) / 1e12,
            "path": "fused" if (n_in, n_hid, nh) == (16, 256, 3) else "one GEMM launch per layer"}


def main(argv=None) -> int:
    """Train the surrogate on the GPU and save it:
    python -m ice3gb.surrogate --points 16777216 --epochs 12 --out PATH
    (--hidden / --layers for another width or depth, --time-rows N to time
    the network on N rows)"""
    import argparse
    import json
    import time
    ap = argparse.ArgumentParser()
    ap.add_argument("--points", type=int, default=1 << 24)
    ap.add_argument("--eval-points", type=int, default=1 << 20)
    ap.add_argument("--epochs", type=int, default=12)
    ap.add_argument("--batch", type=int, default=16384)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--hidden", type=int, default=256)
    ap.add_argument("--layers", type=int, default=3)
    ap.add_argument("--time-rows", type=int, default=0)
    ap.add_argument("--out", default=DEFAULT_PATH)
    ap.add_argument("--report", default=None)
    a = ap.parse_args(argv)
    t0 = time.time()
    raw, tgt = training_set(a.points, seed=1000)
    t1 = time.time()
    sur = SlowSurrogate(seed=a.seed, n_hidden=a.hidden, n_hidden_layers=a.layers)
    sur.train(raw, tgt, epochs=a.epochs, batch=a.batch, lr=a.lr, seed=a.seed)
    torch.cuda.synchronize()
    t2 = time.time()
    ev_raw, ev_tgt = training_set(a.eval_points, seed=900000)
    rep = {"hidden": a.hidden, "layers": a.layers, "train_points": a.points, "epochs": a.epochs, "batch": a.batch,
           "lr": a.lr,
           "sample_s": t1 - t0, "train_s": t2 - t1, "history": sur.history,
           "held_out": sur.rate_errors(ev_raw, ev_tgt),
           "held_out_inside_envelope": float(sur.inside(sur.standardize(ev_raw)).double().mean())}
    if a.time_rows:
        rep["inference"] = time_inference(sur, a.time_rows)
    sur.save(a.out)
    print(json.dumps(rep, indent=1))
    if a.report:
        with open(a.report, "w") as fh:
            json.dump(rep, fh, indent=1)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
