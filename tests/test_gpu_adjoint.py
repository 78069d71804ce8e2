"""Adjoints on the GPU: the ice_adjust and sedimentation vector-Jacobian
products behind torch.autograd (ice3gb.autodiff) against centred finite
differences of the device forward (h = 1e-7, relative directions) on the
256x256x90 adjoint configuration, and the device adjoint kernels against
the host builds of the same code."""
import numpy as np
import pytest
import torch

import test_adjoint_host as H
from test_adjoint_host import lib  # noqa: F401  (host build of the adjoint, a fixture)

pytestmark = pytest.mark.gpu

DT = 50.0
TARGETS = ("t", "rv_out", "rc_out", "ri_out", "cldfr")


def _dev(x):
    return {k: torch.as_tensor(np.ascontiguousarray(v)).cuda() for k, v in x.items()}


def _ia_state(nij, seed, mf=False):
    x = H._state(nij, seed=seed, mf=mf)
    x["sigqsat"] = x["sigqsat"][0].copy()          # per column, as the component takes it
    return x


def test_ice_adjust_autograd_matches_finite_differences():
    """Directional derivative of <g, (T, rv, rc, ri, cldfr)> per grid point,
    backward pass vs centred difference; points where the forward is not
    smooth across the stencil (the jump of CB02 at zero cloud fraction) are
    left out and must carry a small share (sigqsat, a per-column input, is
    held fixed here; its gradient is checked against the host build)."""
    from ice3gb import IceAdjust
    from ice3gb.autodiff import ice_adjust
    ia = IceAdjust()
    x = _dev(_ia_state(256 * 256, seed=1))
    gen = torch.Generator(device="cuda").manual_seed(3)
    shape = x["th"].shape
    g = {k: torch.randn(shape, generator=gen, dtype=torch.float64, device="cuda") for k in TARGETS}
    xr = {k: v.clone().requires_grad_(True) for k, v in x.items()}
    y = ice_adjust(ia, DT, **xr)
    sum((y[k] * g[k]).sum() for k in TARGETS).backward()
    dx = {k: torch.randn(v.shape, generator=gen, dtype=torch.float64, device="cuda") * v.abs() for k, v in x.items()}
    dx["sigqsat"].zero_()
    ad = sum(xr[k].grad * dx[k] for k in x if k != "sigqsat").cpu().numpy().ravel()
    h = 1e-7
    with torch.no_grad():
        js = []
        for sgn in (1.0, 0.0, -1.0):
            ys = ice_adjust(ia, DT, **{k: v + sgn * h * dx[k] for k, v in x.items()})
            js.append(sum(g[k] * ys[k] for k in TARGETS).cpu().numpy().ravel())
    jp, j0, jm = js
    fd = (jp - jm) / (2 * h)
    smooth = H.smooth_points(jp, j0, jm, h)
    H.assert_mostly_smooth(ad, smooth)
    a, f = ad[smooth].sum(), fd[smooth].sum()
    assert abs(a - f) <= 1e-6 * np.abs(ad[smooth]).sum(), (a, f)


def test_ice_adjust_vjp_device_matches_host_build(lib):  # noqa: F811
    from ice3gb import IceAdjust
    from ice3gb.autodiff import ice_adjust
    ia = IceAdjust()
    xn = _ia_state(32 * 32, seed=2, mf=True)
    x = {k: v.clone().requires_grad_(True) for k, v in _dev(xn).items()}
    rng = np.random.default_rng(4)
    gn = {k: rng.standard_normal(xn["th"].shape) for k in H.OUT}
    y = ice_adjust(ia, DT, **x)
    sum((y[k] * torch.as_tensor(gn[k]).cuda()).sum() for k in H.OUT).backward()
    x3 = dict(xn)
    x3["sigqsat"] = np.broadcast_to(xn["sigqsat"][None, :], xn["th"].shape).copy()
    ref = H.vjp(lib, ia.table, x3, gn)
    for k in H.IN:
        got = x[k].grad.cpu().numpy()
        r = ref[k].reshape(xn["th"].shape)
        if k == "sigqsat":
            r = r.sum(axis=0)                       # per-column sigqsat: summed over levels
        tol = 1e-9 * (np.abs(r) + np.abs(r).max() * 1e-6)
        bad = np.abs(got - r) > tol
        assert bad.mean() < 1e-3, f"{k}: {int(bad.sum())} points differ"


def test_sedimentation_autograd_matches_finite_differences():
    from ice3gb import Sedimentation
    from ice3gb.autodiff import SED_IN, sedimentation
    for semantics in ("phyex", "jax"):
        sed = Sedimentation(table="phyex", semantics=semantics)
        x = _dev(H._sed_state(256 * 256, seed=5))
        gen = torch.Generator(device="cuda").manual_seed(7)
        outs = ("rcs", "rrs", "ris", "rss", "rgs", "inprc", "inprr", "inpri", "inprs", "inprg")
        with torch.no_grad():
            y0 = sedimentation(sed, DT, **x)
        g = {k: torch.randn(y0[k].shape, generator=gen, dtype=torch.float64, device="cuda") /
             max(float(y0[k].abs().max()), 1e-300) for k in outs}
        xr = {k: v.clone().requires_grad_(True) for k, v in x.items()}
        y = sedimentation(sed, DT, **xr)
        sum((y[k] * g[k]).sum() for k in outs).backward()
        dx = {k: torch.randn(v.shape, generator=gen, dtype=torch.float64, device="cuda") * v.abs()
              for k, v in x.items()}
        ad = sum(float((xr[k].grad * dx[k]).sum()) for k in SED_IN)
        scale = sum(float((xr[k].grad * dx[k]).abs().sum()) for k in SED_IN)
        h = 1e-7
        with torch.no_grad():
            yp = sedimentation(sed, DT, **{k: v + h * dx[k] for k, v in x.items()})
            ym = sedimentation(sed, DT, **{k: v - h * dx[k] for k, v in x.items()})
        fd = sum(float((g[k] * (yp[k] - ym[k])).sum()) for k in outs) / (2 * h)
        assert abs(ad - fd) <= 1e-6 * scale, (semantics, ad, fd, scale)


def test_adjoints_match_reference_differences():
    """The device adjoints through torch.autograd against centred differences
    of the reference's own IceAdjustJAX and sedimentation_stat (FP64, h = 1e-7;
    tests/golden/adjoint_fd.npz): every smooth point within 1e-6."""
    from conftest import load_golden
    from ice3gb import IceAdjust, Sedimentation
    from ice3gb.autodiff import ice_adjust, sedimentation
    g = load_golden("adjoint_fd")
    x = {k: torch.as_tensor(g[f"ia_x_{k}"]).cuda().requires_grad_(True) for k in H.IN}
    y = ice_adjust(IceAdjust(), DT, **x)
    sum((y[k] * torch.as_tensor(g[f"ia_g_{k}"]).cuda()).sum() for k in TARGETS).backward()
    ad = sum(x[k].grad.cpu().numpy() * g[f"ia_dx_{k}"] for k in H.IN).ravel()
    H.reference_ice_adjust_check(ad, g)

    sin = ("rhodref", "dzz", "pabs", "tht") + H.SRC
    sx = {k: torch.as_tensor(g[f"sed_x_{k}"]).cuda().requires_grad_(True) for k in sin}
    ys = sedimentation(Sedimentation(semantics="jax"), DT, **sx)
    loss = sum((ys[k] * torch.as_tensor(g[f"sed_g_{k}"]).cuda()).sum() for k in H.SRC + H.INPR)
    loss.backward()
    ad = sum((sx[k].grad.cpu().numpy() * g[f"sed_dx_{k}"]).sum(axis=0) for k in sin)
    H.reference_sedimentation_check(ad, g)
