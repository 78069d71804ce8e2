"""Seeded synthetic atmospheric states for the ICE3 hot path.

Column layout [nk][nij] (horizontal index fastest, k = 0 at the surface), FP64.
The distributions follow the workload definitions of the benchmark:

* surface pressure ps ~ U[990, 1010] hPa per column; levels p_k = ps * eta_k
  with eta geometric from 1 at the surface to 10 hPa / ps at the top;
* z from the inverse of the ICAO standard atmosphere, T = 288 K - 6.5 K/km z
  floored at 216.65 K above 11 km, plus N(0, 1 K) noise;
* exn = exn_ref = (p/P00)**(RD/CPD), th = T/exn, rho = p/(RD T), dzz from the
  hypsometric thickness between consecutive levels (top level repeats the
  thickness below it);
* rv = RH * qsat with RH ~ U[0.3, 1.05], qsat w.r.t. liquid above 273.15 K and
  ice below (saturation formula and constants of the constants table);
* rc, ri ~ LogNormal(ln 1e-5, 1), each zero with probability 0.5, ri = 0 where
  T >= 268 K; sigs ~ U[1e-6, 1e-4]; sigqsat = 0.02 per column;
  cf_mf = rc_mf = ri_mf = 0;
* sources S = x_t / dt (th/dt, r/dt): the PHYEX convention for a step with
  no other tendency (the external tendency S - x_t/dt of
  mode_ice4_stepping.F90:151-158 is then zero);
* with ``precip=True`` also rr, rs, rg ~ LogNormal(ln 1e-5, 1.5) each zero
  with probability 0.6, cloud fraction ~ U[0, 1] where rc + ri > 0,
  ci_t = hlc_* = hli_* = 0, sea = town = 0.

Generation runs with torch on the requested device (one seeded generator),
so full-size states are built directly in GPU memory.
"""
from __future__ import annotations

import math
from typing import Dict, Mapping, Optional

import torch

from .constants import externals_from

G0 = 9.80665
ISA_P0, ISA_T0, ISA_L, ISA_T11 = 101325.0, 288.15, 0.0065, 216.65


def _lognormal(gen, shape, median, sigma, device):
    z = torch.randn(shape, generator=gen, device=device, dtype=torch.float64)
    return median * torch.exp(sigma * z)


def make_state(nij: int, nk: int = 90, seed: int = 0, precip: bool = False,
               device="cpu", phyex: Optional[Mapping] = None, dt: float = 50.0) -> Dict[str, torch.Tensor]:
    """Return a dict of [nk, nij] float64 tensors (2-D per-column fields are [nij])."""
    ext = externals_from(phyex)
    RD, CPD, P00, EPSILO = (float(ext[k]) for k in ("RD", "CPD", "P00", "EPSILO"))
    ALPW, BETAW, GAMW = (float(ext[k]) for k in ("ALPW", "BETAW", "GAMW"))
    ALPI, BETAI, GAMI = (float(ext[k]) for k in ("ALPI", "BETAI", "GAMI"))
    dev = torch.device(device)
    gen = torch.Generator(device=dev)
    gen.manual_seed(int(seed))
    f64 = dict(dtype=torch.float64, device=dev)

    def uni(shape, lo, hi):
        return lo + (hi - lo) * torch.rand(shape, generator=gen, **f64)

    ps = uni((nij,), 990e2, 1010e2)
    frac = torch.arange(nk, **f64) / max(nk - 1, 1)
    # p_k = ps * (1000 Pa / ps) ** (k / (nk-1))
    p = ps[None, :] * torch.exp(frac[:, None] * torch.log(1000.0 / ps[None, :]))
    # ISA inverse
    p11 = ISA_P0 * (ISA_T11 / ISA_T0) ** (G0 / (RD * ISA_L))
    z_trop = ISA_T0 / ISA_L * (1.0 - (p / ISA_P0) ** (RD * ISA_L / G0))
    z_strat = 11000.0 + RD * ISA_T11 / G0 * torch.log(p11 / p)
    z = torch.where(p >= p11, z_trop, z_strat)
    t = torch.clamp(288.0 - 6.5e-3 * z, min=216.65) + torch.randn((nk, nij), generator=gen, **f64)
    exn = (p / P00) ** (RD / CPD)
    th = t / exn
    rho = p / (RD * t)
    dz = torch.empty_like(p)
    dz[:-1] = RD * 0.5 * (t[:-1] + t[1:]) / G0 * torch.log(p[:-1] / p[1:])
    dz[-1] = dz[-2] if nk > 1 else 100.0
    es_w = torch.exp(ALPW - BETAW / t - GAMW * torch.log(t))
    es_i = torch.exp(ALPI - BETAI / t - GAMI * torch.log(t))
    e = torch.where(t > 273.15, es_w, es_i)
    qsat = EPSILO * e / (p - e)
    rv = uni((nk, nij), 0.3, 1.05) * qsat
    rc = _lognormal(gen, (nk, nij), 1e-5, 1.0, dev)
    rc = torch.where(torch.rand((nk, nij), generator=gen, **f64) < 0.5, torch.zeros_like(rc), rc)
    ri = _lognormal(gen, (nk, nij), 1e-5, 1.0, dev)
    ri = torch.where(torch.rand((nk, nij), generator=gen, **f64) < 0.5, torch.zeros_like(ri), ri)
    ri = torch.where(t >= 268.0, torch.zeros_like(ri), ri)
    sigs = uni((nk, nij), 1e-6, 1e-4)
    zeros = torch.zeros((nk, nij), **f64)
    st = {
        "sigqsat": torch.full((nij,), 0.02, **f64),
        "pabs": p, "sigs": sigs, "th": th, "exn": exn, "exn_ref": exn.clone(),
        "rho_dry_ref": rho, "rv": rv, "rc": rc, "ri": ri,
        "cf_mf": zeros.clone(), "rc_mf": zeros.clone(), "ri_mf": zeros.clone(),
        "rvs": rv / dt, "rcs": rc / dt, "ris": ri / dt, "ths": th / dt,
        "dzz": dz, "t": t,
    }
    if precip:
        for name in ("rr", "rs", "rg"):
            r = _lognormal(gen, (nk, nij), 1e-5, 1.5, dev)
            st[name] = torch.where(torch.rand((nk, nij), generator=gen, **f64) < 0.6, torch.zeros_like(r), r)
        cf = uni((nk, nij), 0.0, 1.0)
        st["cldfr"] = torch.where(rc + ri > 0, cf, torch.zeros_like(cf))
        for name in ("rr", "rs", "rg"):
            st[name + "s"] = st[name] / dt
        for name in ("ci_t", "hlc_hrc", "hlc_hcf", "hli_hri", "hli_hcf"):
            st[name] = zeros.clone()
        st["sea"] = torch.zeros((nij,), **f64)
        st["town"] = torch.zeros((nij,), **f64)
    else:
        for name in ("rr", "rs", "rg"):
            st[name] = zeros.clone()
    return st


def rain_ice_state(st: Dict[str, torch.Tensor]) -> Dict[str, torch.Tensor]:
    """Map a make_state(..., precip=True) dict to the RainIce state keys
    (the RainIceJAX state-dict names, src/ice3/jax/rain_ice.py:209-260)."""
    return {
        "exn": st["exn"], "dzz": st["dzz"], "rhodref": st["rho_dry_ref"], "exnref": st["exn_ref"],
        "pres": st["pabs"], "cldfr": st["cldfr"], "sigs": st["sigs"],
        "th_t": st["th"], "rv_t": st["rv"], "rc_t": st["rc"], "rr_t": st["rr"],
        "ri_t": st["ri"], "rs_t": st["rs"], "rg_t": st["rg"], "ci_t": st["ci_t"],
        "hlc_hrc": st["hlc_hrc"], "hlc_hcf": st["hlc_hcf"], "hli_hri": st["hli_hri"], "hli_hcf": st["hli_hcf"],
        "ths": st["ths"], "rvs": st["rvs"], "rcs": st["rcs"], "rrs": st["rrs"], "ris": st["ris"],
        "rss": st["rss"], "rgs": st["rgs"], "sea": st["sea"], "town": st["town"],
    }
