"""Torch-facing drop-in components over libice3gb.so.

* ``IceAdjust(phyex)(**20 named fields, timestep)`` -> the 16-tuple of
  ``IceAdjustJAX.__call__`` (src/ice3/jax/ice_adjust.py:139-230).
* ``RainIce(constants)(state, dt, lsedim_after=..., ...)`` -> ``(state,
  diagnostics)`` like ``RainIceJAX.__call__`` (src/ice3/jax/rain_ice.py:181).
  The step follows PHYEX RAIN_ICE: the returned state carries the updated
  sources ths/rvs/rcs/rrs/ris/rss/rgs and ci_t (the *_t fields are the
  time-t prognostic inputs and are returned unchanged), the diagnostics the
  instantaneous precipitation inpr{c,r,i,s,g}, evap3d and rainfr.
* ``Sedimentation(...)(...)`` ~ ``sedimentation_stat``
  (src/ice3/jax/stencils/sedimentation.py:58).

Fields are float64 torch tensors on the current CUDA device.  Vertical
layout: "kij" = [nk, nij...] (k slowest, k = 0 at the surface, the ABI's own
order) or "jax" = (ngpblks, nproma, nflevg) as the reference JAX stores it
(transposed on the way in and out).  NumPy arrays are accepted too: they go
through the host-buffer entry points and NumPy arrays come back.
"""
from __future__ import annotations

import ctypes
from typing import Any, Dict, Mapping, Optional, Tuple

import numpy as np
import torch

from . import _abi
from .constants import ConstantsTable, build_table

IA_INPUTS = ("sigqsat", "pabs", "sigs", "th", "exn", "exn_ref", "rho_dry_ref", "rv", "rc", "ri", "rr", "rs", "rg",
             "cf_mf", "rc_mf", "ri_mf")
IA_INOUT = ("rvs", "rcs", "ris", "ths")
IA_OUTPUTS = ("t", "rv_out", "rc_out", "ri_out", "cldfr", "hlc_hrc", "hlc_hcf", "hli_hri", "hli_hcf", "cph", "lv",
              "ls")


def _stream_ptr() -> int:
    return torch.cuda.current_stream().cuda_stream


class Ice3Handle:
    """One constants table uploaded on the current CUDA device."""

    def __init__(self, table: ConstantsTable):
        self.lib = _abi.load()
        self.table = table
        h = ctypes.c_void_p()
        _abi.check(self.lib.ice3gb_create(ctypes.byref(table.consts), ctypes.byref(table.luts), ctypes.byref(h)),
                   None, "ice3gb_create")
        self.h = h

    def __del__(self):
        h = getattr(self, "h", None)
        if h is not None and h.value:
            try:
                self.lib.ice3gb_destroy(h)
            except Exception:
                pass
            self.h = None

    def status(self) -> int:
        bits = ctypes.c_uint32(0)
        rc = self.lib.ice3gb_status(self.h, ctypes.c_void_p(_stream_ptr()), ctypes.byref(bits))
        if rc not in (0, -6):
            _abi.check(rc, self.h, "ice3gb_status")
        return bits.value


def _as_device_f64(x, like: Optional[torch.Tensor] = None) -> torch.Tensor:
    if isinstance(x, torch.Tensor):
        t = x
    else:
        t = torch.as_tensor(np.asarray(x, dtype=np.float64))
    dev = like.device if like is not None else torch.device("cuda", torch.cuda.current_device())
    if t.device != dev or t.dtype != torch.float64:
        t = t.to(device=dev, dtype=torch.float64)
    return t.contiguous()


def _ptr(t: Optional[torch.Tensor]):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


class IceAdjust:
    """Drop-in for ``IceAdjustJAX`` (src/ice3/jax/ice_adjust.py:40-230)."""

    def __init__(self, phyex: Any = None, jit: bool = True, table: str = "jax"):
        # `jit` is accepted for signature compatibility; the kernel is compiled ahead of time.
        self.table = build_table(phyex, table=table)
        self.constants = self.table.values
        self._handle: Optional[Ice3Handle] = None

    @property
    def handle(self) -> Ice3Handle:
        if self._handle is None:
            self._handle = Ice3Handle(self.table)
        return self._handle

    @property
    def ocnd2(self) -> bool:
        return self.table.values["OCND2"] != 0.0

    def __call__(self, sigqsat, pabs, sigs, th, exn, exn_ref, rho_dry_ref, rv, rc, ri, rr, rs, rg, cf_mf, rc_mf,
                 ri_mf, rvs, rcs, ris, ths, timestep: float, return_srcs: bool = False, zz=None,
                 ice_cld_wgt=None) -> Tuple:
        """The 16-tuple of IceAdjustJAX; with ``return_srcs`` a 17th element,
        PSRCS (s'r_c'/sigma_s^2, the second-order flux term the Fortran
        ICE_ADJUST returns, ice_adjust.F90:468).

        With OCND2 set in the constants table (separate liquid and ice
        clouds, condensation.F90:373-395, :588-637) the fields are laid out
        [nk, ...] with k = 0 at the surface, ``zz`` (height of the levels, m,
        same shape) and ``ice_cld_wgt`` (one value per column) are required,
        and five more elements follow: icldfr, wcldfr, ssio, ssiu, ifr
        (ice_adjust.F90:177-183)."""
        args = dict(sigqsat=sigqsat, pabs=pabs, sigs=sigs, th=th, exn=exn, exn_ref=exn_ref,
                    rho_dry_ref=rho_dry_ref, rv=rv, rc=rc, ri=ri, rr=rr, rs=rs, rg=rg, cf_mf=cf_mf, rc_mf=rc_mf,
                    ri_mf=ri_mf, rvs=rvs, rcs=rcs, ris=ris, ths=ths)
        if self.ocnd2:
            if zz is None or ice_cld_wgt is None:
                raise ValueError("OCND2 needs zz and ice_cld_wgt")
            args.update(zz=zz, ice_cld_wgt=ice_cld_wgt)
        if isinstance(pabs, np.ndarray):
            return self._call_host(args, float(timestep), return_srcs)
        ref = pabs
        shape = tuple(ref.shape)
        dev = {k: _as_device_f64(v, ref) for k, v in args.items()}
        for k, v in dev.items():
            if k not in ("sigqsat", "ice_cld_wgt") and tuple(v.shape) != shape:
                raise ValueError(f"{k} has shape {tuple(v.shape)}, expected {shape}")
        nij, nk, sig3d = self._geometry(shape, tuple(dev["sigqsat"].shape))
        outs = {k: torch.empty(shape, dtype=torch.float64, device=ref.device) for k in IA_OUTPUTS}
        io = {k: dev[k].clone() for k in IA_INOUT}
        f = _abi.IceAdjustFields()
        for k in IA_INPUTS:
            setattr(f, k, _ptr(dev[k]))
        for k, v in {**io, **outs}.items():
            setattr(f, k, _ptr(v))
        f.sigqsat_3d = sig3d
        srcs = torch.empty(shape, dtype=torch.float64, device=ref.device) if return_srcs else None
        f.srcs = _ptr(srcs)
        extra = ()
        if self.ocnd2:
            self._check_ocnd2(shape, nij, tuple(dev["ice_cld_wgt"].shape))
            f.zz, f.ice_cld_wgt = _ptr(dev["zz"]), _ptr(dev["ice_cld_wgt"])
            extra = tuple(torch.empty(shape, dtype=torch.float64, device=ref.device) for _ in _abi.OCND2_OUTPUTS)
            for k, v in zip(_abi.OCND2_OUTPUTS, extra):
                setattr(f, k, _ptr(v))
        h = self.handle
        _abi.check(h.lib.ice3gb_ice_adjust(h.h, nij, nk, float(timestep), ctypes.byref(f),
                                           ctypes.c_void_p(_stream_ptr())), h.h, "ice3gb_ice_adjust")
        res = tuple(outs[k] for k in IA_OUTPUTS) + tuple(io[k] for k in IA_INOUT)
        return (res + (srcs,) if return_srcs else res) + extra

    def _geometry(self, shape, sig_shape):
        if self.ocnd2:
            # levels are needed (layer thickness): [nk, ...] whatever sigqsat's shape
            if len(shape) < 2:
                raise ValueError("OCND2 needs fields shaped [nk, ...]")
            nij = int(np.prod(shape[1:]))
            if tuple(sig_shape) == tuple(shape):
                return nij, int(shape[0]), 1
            if int(np.prod(sig_shape)) == nij:
                return nij, int(shape[0]), 0
            raise ValueError(f"sigqsat shape {sig_shape} matches neither the fields {shape} nor one level")
        return self._geometry_any(shape, sig_shape)

    @staticmethod
    def _check_ocnd2(shape, nij, wgt_shape):
        if int(np.prod(wgt_shape)) != nij:
            raise ValueError(f"ice_cld_wgt has shape {wgt_shape}, expected one value per column ({nij})")

    @staticmethod
    def _geometry_any(shape, sig_shape):
        n = int(np.prod(shape))
        if tuple(sig_shape) == tuple(shape):
            return n, 1, 1                       # full 3-D sigqsat: pointwise, any layout
        if len(shape) >= 2 and int(np.prod(sig_shape)) == int(np.prod(shape[1:])):
            return int(np.prod(shape[1:])), int(shape[0]), 0   # [nk, ...] with per-column sigqsat
        raise ValueError(f"sigqsat shape {sig_shape} matches neither the fields {shape} nor one level")

    def _call_host(self, args: Dict[str, np.ndarray], dt: float, return_srcs: bool = False) -> Tuple:
        shape = args["pabs"].shape
        host = {k: np.ascontiguousarray(np.asarray(v, dtype=np.float64)) for k, v in args.items()}
        nij, nk, sig3d = self._geometry(shape, host["sigqsat"].shape)
        io = {k: host[k].copy() for k in IA_INOUT}
        outs = {k: np.empty(shape) for k in IA_OUTPUTS}
        f = _abi.IceAdjustFields()
        for k in IA_INPUTS:
            setattr(f, k, host[k].ctypes.data_as(ctypes.c_void_p))
        for k, v in {**io, **outs}.items():
            setattr(f, k, v.ctypes.data_as(ctypes.c_void_p))
        f.sigqsat_3d = sig3d
        srcs = np.empty(shape) if return_srcs else None
        if return_srcs:
            f.srcs = srcs.ctypes.data_as(ctypes.c_void_p)
        extra = ()
        if self.ocnd2:
            self._check_ocnd2(shape, nij, host["ice_cld_wgt"].shape)
            f.zz = host["zz"].ctypes.data_as(ctypes.c_void_p)
            f.ice_cld_wgt = host["ice_cld_wgt"].ctypes.data_as(ctypes.c_void_p)
            extra = tuple(np.empty(shape) for _ in _abi.OCND2_OUTPUTS)
            for k, v in zip(_abi.OCND2_OUTPUTS, extra):
                setattr(f, k, v.ctypes.data_as(ctypes.c_void_p))
        h = self.handle
        _abi.check(h.lib.ice3gb_ice_adjust_host(h.h, nij, nk, dt, ctypes.byref(f), ctypes.c_void_p(_stream_ptr())),
                   h.h, "ice3gb_ice_adjust_host")
        res = tuple(outs[k] for k in IA_OUTPUTS) + tuple(io[k] for k in IA_INOUT)
        return (res + (srcs,) if return_srcs else res) + extra


# RainIceJAX state keys -> ABI fields (src/ice3/jax/rain_ice.py:209-260,
# tests/components/test_rain_ice_jax.py:84-104)
RI_STATE_IN = {"exn": "exn", "dzz": "dzz", "rhodref": "rhodref", "exnref": "exnref", "pres": "pabs",
               "cldfr": "cldfr", "sigs": "sigs", "th_t": "tht", "rv_t": "rvt", "rc_t": "rct", "rr_t": "rrt",
               "ri_t": "rit", "rs_t": "rst", "rg_t": "rgt"}
RI_STATE_INOUT = {"ci_t": "cit", "hlc_hrc": "hlc_hrc", "hlc_hcf": "hlc_hcf", "hli_hri": "hli_hri",
                  "hli_hcf": "hli_hcf", "ths": "ths", "rvs": "rvs", "rcs": "rcs", "rrs": "rrs", "ris": "ris",
                  "rss": "rss", "rgs": "rgs"}
RI_DIAG3 = ("evap3d", "rainfr")
RI_DIAG2 = ("inprc", "inprr", "inpri", "inprs", "inprg", "indep")


class RainIce:
    """Drop-in for ``RainIceJAX`` (src/ice3/jax/rain_ice.py:20-420), PHYEX semantics.

    ``constants``: a ``Phyex(...).to_externals()`` dict (as RainIceJAX takes),
    a ``Phyex`` object, or None for the shipped AROME table.
    ``table``: "phyex" (default: the reference's table with the Fortran values
    where the Python initialisation diverges, see ice3gb.constants) or "jax".
    ``sedimentation``: "phyex" (Fortran, default) or "jax" (the reference JAX
    sedimentation_stat scaling); see include/ice3gb.h.
    """

    def __init__(self, constants: Any = None, table: str = "phyex", sedimentation: str = "phyex",
                 layout: str = "kij"):
        if sedimentation not in ("phyex", "jax"):
            raise ValueError("sedimentation must be 'phyex' or 'jax'")
        if layout not in ("kij", "jax"):
            raise ValueError("layout must be 'kij' or 'jax'")
        self.table = build_table(constants, table=table)
        self.constants = self.table.values
        self.sed_jax = 1 if sedimentation == "jax" else 0
        self.layout = layout
        self._handle: Optional[Ice3Handle] = None

    @property
    def handle(self) -> Ice3Handle:
        if self._handle is None:
            self._handle = Ice3Handle(self.table)
        return self._handle

    def _to_kij(self, t: torch.Tensor) -> torch.Tensor:
        if self.layout == "jax" and t.dim() == 3:
            g, p, z = t.shape
            return t.permute(2, 0, 1).reshape(z, g * p).contiguous()
        return t.contiguous()

    def _from_kij(self, t: torch.Tensor, like_shape) -> torch.Tensor:
        if self.layout == "jax" and len(like_shape) == 3:
            g, p, z = like_shape
            return t.reshape(z, g, p).permute(1, 2, 0).contiguous()
        return t

    def prepare(self, state: Mapping[str, Any], with_fluxes: bool = False) -> Dict[str, Any]:
        """The ABI field set of one call: {"f": RainIceFields, "fields": in/in-out
        tensors (in-out ones cloned), "diag": outputs, "nij", "nk", "shape",
        "host"}; the tensors must stay alive while the call runs."""
        ref = state["th_t"]
        host = isinstance(ref, np.ndarray)
        if host:
            ref_t = torch.as_tensor(np.ascontiguousarray(ref, dtype=np.float64))
        else:
            ref_t = ref
        shape = tuple(ref_t.shape)

        def get(key, default=None):
            v = state.get(key, default)
            if v is None:
                return None
            if host:
                return torch.as_tensor(np.ascontiguousarray(np.asarray(v, dtype=np.float64)))
            return _as_device_f64(v, ref_t)

        fields: Dict[str, torch.Tensor] = {}
        for key, abi in RI_STATE_IN.items():
            v = get(key)
            if v is None:
                if key == "exnref":
                    v = get("exn")
                elif key == "cldfr":
                    v = torch.zeros_like(ref_t, dtype=torch.float64, device=ref_t.device)
                else:
                    raise KeyError(f"state is missing {key!r}")
            fields[abi] = self._to_kij(v)
        nk, nij = fields["tht"].shape[0], int(np.prod(fields["tht"].shape[1:]))
        for key, abi in RI_STATE_INOUT.items():
            v = get(key)
            if v is None:
                if key.startswith("hl") or key == "ci_t" or key.endswith("s"):
                    v = torch.zeros(shape, dtype=torch.float64, device=ref_t.device)
            fields[abi] = self._to_kij(v).clone()
        hail = self.table.values["NRR"] == 7.0
        if hail:
            # NRR = 7: hail at t and its source (RainIceJAX's state has no hail;
            # the keys follow its naming, rh_t / rhs)
            rh = get("rh_t")
            if rh is None:
                raise KeyError("state is missing 'rh_t' (NRR = 7)")
            fields["rht"] = self._to_kij(rh)
            rhs = get("rhs")
            fields["rhs"] = (self._to_kij(rhs) if rhs is not None
                             else torch.zeros((nk, nij), dtype=torch.float64, device=ref_t.device)).clone()
        if self.table.values["OCND2"] != 0.0:
            # OCND2: the ice_adjust OCND2 outputs of the same state (IceAdjust's
            # five extra outputs), same names
            for k in ("ssio", "ssiu", "ifr", "icldfr"):
                v = get(k)
                if v is None:
                    raise KeyError(f"state is missing {k!r} (OCND2)")
                fields[k] = self._to_kij(v)
        sea, town = get("sea"), get("town")
        if (sea is None) != (town is None):
            raise ValueError("sea and town must be given together")
        if sea is not None:
            sea, town = sea.reshape(-1).contiguous(), town.reshape(-1).contiguous()
        dev = fields["tht"].device
        diag = {k: torch.empty((nk, nij), dtype=torch.float64, device=dev) for k in RI_DIAG3}
        diag.update({k: torch.empty((nij,), dtype=torch.float64, device=dev) for k in RI_DIAG2})
        if with_fluxes:
            diag.update({k: torch.empty((nk, nij), dtype=torch.float64, device=dev)
                         for k in ("fpr_c", "fpr_r", "fpr_i", "fpr_s", "fpr_g")})
        if hail:
            diag["inprh"] = torch.empty((nij,), dtype=torch.float64, device=dev)
            if with_fluxes:
                diag["fpr_h"] = torch.empty((nk, nij), dtype=torch.float64, device=dev)
        f = _abi.RainIceFields()
        for k, v in fields.items():
            setattr(f, k, _ptr(v))
        for k, v in diag.items():
            setattr(f, k, _ptr(v))
        f.sea, f.town = _ptr(sea), _ptr(town)
        return {"f": f, "fields": fields, "diag": diag, "sea": sea, "town": town, "nij": nij, "nk": nk,
                "shape": shape, "host": host}

    def __call__(self, state: Mapping[str, Any], dt: float, lsedim_after: bool = False, ldeposc: bool = False,
                 ldsoft: bool = False, lfeedbackt: bool = True, max_iterations: Optional[int] = None,
                 with_fluxes: bool = False, surrogate: Any = None):
        """``surrogate``: an ``ice3gb.surrogate.SlowSurrogate`` to take the
        ICE4_SLOW rates from the learned network (CUDA tensors only); its
        counters of the call go to ``self.surrogate_stats``."""
        # ldsoft is accepted for signature compatibility: the soft/hard passes are
        # decided inside the ICE4 sub-stepping as in PHYEX.
        c = self.prepare(state, with_fluxes)
        f, fields, diag, nij, nk, shape, host = (c["f"], c["fields"], c["diag"], c["nij"], c["nk"], c["shape"],
                                                 c["host"])
        opt = _abi.RainIceOptions(int(bool(lsedim_after)), int(bool(ldeposc)), int(bool(lfeedbackt)),
                                  int(max_iterations or 0), self.sed_jax)
        h = self.handle
        sptr = ctypes.c_void_p(_stream_ptr())
        if surrogate is not None:
            if host:
                raise ValueError("the surrogate-assisted rain_ice takes CUDA tensors")
            stats = (ctypes.c_uint64 * _abi.SUR_NSTATS)()
            norm = surrogate.norm_struct()
            _abi.check(h.lib.ice3gb_rain_ice_surrogate(h.h, surrogate.mlp.h, nij, nk, float(dt), ctypes.byref(opt),
                                                       ctypes.byref(f), ctypes.byref(norm), stats, sptr),
                       h.h, "ice3gb_rain_ice_surrogate")
            self.surrogate_stats = dict(zip(_abi.SUR_STATS, (int(v) for v in stats)))
        elif host:
            _abi.check(h.lib.ice3gb_rain_ice_host(h.h, nij, nk, float(dt), ctypes.byref(opt), ctypes.byref(f), sptr),
                       h.h, "ice3gb_rain_ice_host")
        else:
            _abi.check(h.lib.ice3gb_rain_ice(h.h, nij, nk, float(dt), ctypes.byref(opt), ctypes.byref(f), sptr),
                       h.h, "ice3gb_rain_ice")
        out_state = dict(state)
        for key, abi in RI_STATE_INOUT.items():
            v = self._from_kij(fields[abi], shape)
            out_state[key] = v.numpy() if host else v
        if "rhs" in fields:
            v = self._from_kij(fields["rhs"], shape)
            out_state["rhs"] = v.numpy() if host else v
        diagnostics = {}
        for k, v in diag.items():
            v = self._from_kij(v, shape) if v.dim() == 2 else v
            diagnostics[k] = v.numpy() if host else v
        return out_state, diagnostics

    def device_status(self) -> int:
        """Synchronise and return (then clear) the device status bits
        (bit 0: a point reached the sub-step pass cap)."""
        return self.handle.status()


class Sedimentation:
    """Drop-in for ``sedimentation_stat`` (src/ice3/jax/stencils/sedimentation.py:58)."""

    def __init__(self, constants: Any = None, table: str = "jax", semantics: str = "jax"):
        self.table = build_table(constants, table=table)
        self.fortran = 1 if semantics == "phyex" else 0
        self._handle: Optional[Ice3Handle] = None

    @property
    def handle(self) -> Ice3Handle:
        if self._handle is None:
            self._handle = Ice3Handle(self.table)
        return self._handle

    def __call__(self, rhodref, dzz, pabs_t, th_t, rcs, rrs, ris, rss, rgs, sea=None, town=None, dt=None,
                 with_fluxes=True):
        """Fields [nk, nij] on the device; returns (rcs, rrs, ris, rss, rgs,
        fpr_c, fpr_r, fpr_i, fpr_s, fpr_g, inprc, inprr, inpri, inprs, inprg)
        in the reference's order (sedimentation.py:350-352)."""
        dt = float(self.table.values.get("TSTEP", 50.0) if dt is None else dt)
        ref = rhodref
        ins = [_as_device_f64(x, ref) for x in (rhodref, dzz, pabs_t, th_t)]
        src = [_as_device_f64(x, ref).clone() for x in (rcs, rrs, ris, rss, rgs)]
        nk, nij = ins[0].shape[0], int(np.prod(ins[0].shape[1:]))
        fpr = [torch.empty_like(ins[0]) if with_fluxes else None for _ in range(5)]
        inpr = [torch.empty((nij,), dtype=torch.float64, device=ref.device) for _ in range(5)]
        f = _abi.SedimentationFields()
        f.rhodref, f.dzz, f.pabs, f.tht = (_ptr(x) for x in ins)
        if sea is not None:
            sea = _as_device_f64(sea, ref).reshape(-1)
            town = _as_device_f64(town, ref).reshape(-1)
        f.sea, f.town = _ptr(sea), _ptr(town)
        f.rcs, f.rrs, f.ris, f.rss, f.rgs = (_ptr(x) for x in src)
        f.inprc, f.inprr, f.inpri, f.inprs, f.inprg = (_ptr(x) for x in inpr)
        f.fpr_c, f.fpr_r, f.fpr_i, f.fpr_s, f.fpr_g = (_ptr(x) for x in fpr)
        f.fortran_semantics = self.fortran
        h = self.handle
        _abi.check(h.lib.ice3gb_sedimentation(h.h, nij, nk, dt, ctypes.byref(f), ctypes.c_void_p(_stream_ptr())),
                   h.h, "ice3gb_sedimentation")
        return tuple(src) + tuple(fpr) + tuple(inpr)
