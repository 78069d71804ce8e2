"""Differentiable ice_adjust and sedimentation for torch.autograd.

The backward passes are the hand-written adjoint kernels of libice3gb
(ice3gb_ice_adjust_vjp, ice3gb_sedimentation_vjp): recompute-forward, so a
Function saves only its inputs and the backward kernel rebuilds the forward
intermediates it needs.  Device tensors, FP64, layout [nk, nij] as in the
forward components.

    ia = IceAdjust()
    x = {name: tensor.requires_grad_() ...}          # the 20 inputs of IceAdjust
    y = ice_adjust(ia, timestep=50.0, **x)           # dict of the 16 outputs
    (y["t"] * g_t + y["cldfr"] * g_cf).sum().backward()
"""
from __future__ import annotations

import ctypes
from typing import Dict

import torch

from . import _abi
from .components import IceAdjust, Sedimentation, _ptr, _stream_ptr

IA_IN = _abi.IA_IN
IA_OUT = _abi.IA_OUT


def _f64c(t: torch.Tensor) -> torch.Tensor:
    return t.detach().to(dtype=torch.float64).contiguous()


class IceAdjustFunction(torch.autograd.Function):
    """ice_adjust with the hand-written adjoint as its backward."""

    @staticmethod
    def forward(ctx, ia: IceAdjust, timestep: float, *inputs):
        x = dict(zip(IA_IN, (_f64c(t) for t in inputs)))
        outs = ia(**x, timestep=timestep)
        ctx.ia, ctx.timestep = ia, float(timestep)
        ctx.save_for_backward(*[x[k] for k in IA_IN])
        return tuple(outs)

    @staticmethod
    def backward(ctx, *gouts):
        x = dict(zip(IA_IN, ctx.saved_tensors))
        ia: IceAdjust = ctx.ia
        shape = tuple(x["pabs"].shape)
        nij, nk, sig3d = IceAdjust._geometry_any(shape, tuple(x["sigqsat"].shape))
        f = _abi.IceAdjustFields()
        for k in IA_IN:
            setattr(f, k, _ptr(x[k]))
        f.sigqsat_3d = sig3d
        g = _abi.IceAdjustCotangents()
        keep = []
        for k, go in zip(IA_OUT, gouts):
            if go is not None:
                go = _f64c(go)
                keep.append(go)
                setattr(g, k, _ptr(go))
        grads: Dict[str, torch.Tensor] = {}
        gx = _abi.IceAdjustGradients()
        for i, k in enumerate(IA_IN):
            if ctx.needs_input_grad[2 + i]:
                grads[k] = torch.empty_like(x[k])
                setattr(gx, k, _ptr(grads[k]))
        h = ia.handle
        _abi.check(h.lib.ice3gb_ice_adjust_vjp(h.h, nij, nk, ctx.timestep, ctypes.byref(f), ctypes.byref(g),
                                                ctypes.byref(gx), ctypes.c_void_p(_stream_ptr())),
                   h.h, "ice3gb_ice_adjust_vjp")
        return (None, None) + tuple(grads.get(k) for k in IA_IN)


def ice_adjust(ia: IceAdjust, timestep: float, **fields) -> Dict[str, torch.Tensor]:
    """Differentiable IceAdjust call: the 20 named inputs of IceAdjust.__call__
    (device tensors), the 16 outputs returned by name."""
    missing = [k for k in IA_IN if k not in fields]
    if missing:
        raise KeyError(f"missing inputs {missing}")
    outs = IceAdjustFunction.apply(ia, float(timestep), *[fields[k] for k in IA_IN])
    return dict(zip(IA_OUT, outs))


SED_IN = ("rhodref", "dzz", "pabs", "tht", "rcs", "rrs", "ris", "rss", "rgs")
SED_OUT = ("rcs", "rrs", "ris", "rss", "rgs", "fpr_c", "fpr_r", "fpr_i", "fpr_s", "fpr_g",
           "inprc", "inprr", "inpri", "inprs", "inprg")


class SedimentationFunction(torch.autograd.Function):
    """Statistical sedimentation with the hand-written reverse sweep as its
    backward (sea/town, when given, are constants)."""

    @staticmethod
    def forward(ctx, sed: Sedimentation, dt: float, sea, town, *inputs):
        x = dict(zip(SED_IN, (_f64c(t) for t in inputs)))
        outs = sed(x["rhodref"], x["dzz"], x["pabs"], x["tht"], x["rcs"], x["rrs"], x["ris"], x["rss"], x["rgs"],
                   sea=sea, town=town, dt=dt, with_fluxes=True)
        ctx.sed, ctx.dt = sed, float(dt)
        ctx.sea = None if sea is None else _f64c(sea).reshape(-1)
        ctx.town = None if town is None else _f64c(town).reshape(-1)
        ctx.save_for_backward(*[x[k] for k in SED_IN])
        return tuple(outs)

    @staticmethod
    def backward(ctx, *gouts):
        x = dict(zip(SED_IN, ctx.saved_tensors))
        sed: Sedimentation = ctx.sed
        nk, nij = x["rhodref"].shape[0], x["rhodref"][0].numel()
        f = _abi.SedimentationFields()
        for k in SED_IN:
            setattr(f, k, _ptr(x[k]))
        f.sea, f.town = _ptr(ctx.sea), _ptr(ctx.town)
        f.fortran_semantics = sed.fortran
        g = _abi.SedimentationCotangents()
        keep = []
        for k, go in zip(SED_OUT, gouts):
            if go is not None:
                go = _f64c(go)
                keep.append(go)
                setattr(g, k, _ptr(go))
        grads: Dict[str, torch.Tensor] = {}
        gx = _abi.SedimentationGradients()
        for i, k in enumerate(SED_IN):
            if ctx.needs_input_grad[4 + i]:
                grads[k] = torch.empty_like(x[k])
                setattr(gx, k, _ptr(grads[k]))
        h = sed.handle
        _abi.check(h.lib.ice3gb_sedimentation_vjp(h.h, nij, nk, ctx.dt, ctypes.byref(f), ctypes.byref(g),
                                                   ctypes.byref(gx), ctypes.c_void_p(_stream_ptr())),
                   h.h, "ice3gb_sedimentation_vjp")
        return (None, None, None, None) + tuple(grads.get(k) for k in SED_IN)


def sedimentation(sed: Sedimentation, dt: float, sea=None, town=None, **fields) -> Dict[str, torch.Tensor]:
    """Differentiable sedimentation: rhodref, dzz, pabs, tht and the sources
    rcs, rrs, ris, rss, rgs (device tensors [nk, nij]); outputs by name."""
    missing = [k for k in SED_IN if k not in fields]
    if missing:
        raise KeyError(f"missing inputs {missing}")
    outs = SedimentationFunction.apply(sed, float(dt), sea, town, *[fields[k] for k in SED_IN])
    return dict(zip(SED_OUT, outs))
