"""Hand-written adjoint of ice_adjust (ia_point_vjp in ice_adjust_point.cuh,
the code the device adjoint kernel runs), host build, against centred finite
differences of the forward: directional derivatives <gx, dx> vs
(J(x + h dx) - J(x - h dx)) / 2h with J = <g, y(x)>, h = 1e-7, relative
directions dx = N(0,1) |x|.  Cotangents N(0,1) on T, rv, rc, ri and cloud
fraction (the adjoint configuration), then on all 16 outputs."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
DT = 50.0
IN = ("sigqsat", "pabs", "sigs", "th", "exn", "exn_ref", "rho_dry_ref", "rv", "rc", "ri", "rr", "rs", "rg", "cf_mf",
      "rc_mf", "ri_mf", "rvs", "rcs", "ris", "ths")
OUT = ("t", "rv_out", "rc_out", "ri_out", "cldfr", "hlc_hrc", "hlc_hcf", "hli_hri", "hli_hcf", "cph", "lv", "ls", "rvs",
       "rcs", "ris", "ths")


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = tmp_path_factory.mktemp("ia") / "libia_host.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-I",
                    os.path.join(HERE, "..", "include"), os.path.join(HERE, "ice_adjust_point_host.cpp"), "-o",
                    str(out)], check=True)
    return ctypes.CDLL(str(out))


def _ptrs(arrs):
    return (ctypes.c_void_p * len(arrs))(*[None if a is None else a.ctypes.data for a in arrs])


def forward(lib, table, x):
    n = x["th"].size
    ins = [np.ascontiguousarray(x[k], dtype=np.float64).ravel() for k in IN]
    outs = [np.empty(n) for _ in OUT]
    lib.ia_forward_host(ctypes.byref(table.consts), ctypes.c_double(DT), ctypes.c_long(n), _ptrs(ins), _ptrs(outs))
    return dict(zip(OUT, outs))


def vjp(lib, table, x, g):
    n = x["th"].size
    ins = [np.ascontiguousarray(x[k], dtype=np.float64).ravel() for k in IN]
    gout = [None if g.get(k) is None else np.ascontiguousarray(g[k], dtype=np.float64).ravel() for k in OUT]
    gin = [np.empty(n) for _ in IN]
    lib.ia_vjp_host(ctypes.byref(table.consts), ctypes.c_double(DT), ctypes.c_long(n), _ptrs(ins), _ptrs(gout),
                    _ptrs(gin))
    return dict(zip(IN, gin))


def _state(nij, seed, mf=False):
    """Synthetic state for derivative checks.  The synthetic sources are
    exactly S = x/dt, which puts every condensate point with no
    condensation exactly on the kink of the source limiter
    (w = max((r_out - r)/dt, -rs) with both operands equal), where the
    centred difference straddles the kink and returns the mean of the two
    one-sided slopes; the sources are therefore scaled by U[0.5, 1.5]."""
    from ice3gb.state import make_state
    st = {k: v.numpy() for k, v in make_state(nij, 90, seed=seed, precip=True).items()}
    x = {k: st[k] for k in IN if k != "sigqsat"}
    x["sigqsat"] = np.broadcast_to(st["sigqsat"][None, :], st["th"].shape).copy()
    rng = np.random.default_rng(seed + 200)
    for k in ("rvs", "rcs", "ris", "ths"):
        x[k] = x[k] * rng.uniform(0.5, 1.5, x[k].shape)
    if mf:  # exercise the mass-flux branch and the triangle PDF
        rng = np.random.default_rng(seed + 100)
        x["cf_mf"] = rng.uniform(0.0, 0.6, x["th"].shape)
        x["rc_mf"] = x["cf_mf"] * rng.lognormal(np.log(3e-5), 1.0, x["th"].shape)
        x["ri_mf"] = np.where(st["t"] < 263.0, x["cf_mf"] * rng.lognormal(np.log(1e-5), 1.0, x["th"].shape), 0.0)
    return x


def smooth_points(jp, j0, jm, h):
    """Points where the forward is smooth across the +-h stencil: the two
    one-sided differences agree.  ice_adjust is not continuous everywhere
    (CB02 as the reference writes it zeroes the condensate where the clipped
    cloud fraction 0.5 + 0.36 atan(1.55 q1) reaches 0, around q1 = -3.8,
    where the condensate is ~1e-3 sigma, not 0), and a derivative cannot
    represent a jump, so those points are left out of the comparison."""
    dp, dm = (jp - j0) / h, (j0 - jm) / h
    noise = 4e-16 * (np.abs(j0) + np.abs(jp) + np.abs(jm)) / h
    return np.abs(dp - dm) <= 1e-3 * (np.abs(dp) + np.abs(dm)) + 4 * noise


def assert_mostly_smooth(ad, smooth, what="", share=1e-2):
    """The points left out must carry a small share of the derivative (a
    sparse output, nonzero at few points, is allowed a larger share)."""
    w = np.abs(ad)
    assert w[~smooth].sum() <= share * max(w.sum(), 1e-300), f"{what}: {(~smooth).sum()} points excluded"


def directional_check(lib, table, x, g, h=1e-7, seed=0):
    """Per-point directional derivatives: adjoint <gx, dx> and centred
    difference of <g, y>, with the mask of points where the forward is
    smooth across the stencil."""
    rng = np.random.default_rng(seed)
    dx = {k: rng.standard_normal(v.shape) * np.abs(v) for k, v in x.items()}
    gx = vjp(lib, table, x, g)
    ad_pt = sum(gx[k].reshape(v.shape) * dx[k] for k, v in x.items())
    xp = {k: v + h * dx[k] for k, v in x.items()}
    xm = {k: v - h * dx[k] for k, v in x.items()}
    yp, y0, ym = forward(lib, table, xp), forward(lib, table, x), forward(lib, table, xm)
    jp = sum(g[k].ravel() * yp[k] for k in g if g[k] is not None)
    j0 = sum(g[k].ravel() * y0[k] for k in g if g[k] is not None)
    jm = sum(g[k].ravel() * ym[k] for k in g if g[k] is not None)
    fd_pt = (jp - jm) / (2 * h)
    return ad_pt.ravel(), fd_pt, smooth_points(jp, j0, jm, h)


@pytest.mark.parametrize("mf", [False, True])
def test_ice_adjust_adjoint_matches_finite_differences(lib, mf):
    from ice3gb.constants import build_table
    table = build_table(table="jax")
    x = _state(32 * 32, seed=3, mf=mf)
    rng = np.random.default_rng(11)
    g = {k: rng.standard_normal(x["th"].shape) for k in ("t", "rv_out", "rc_out", "ri_out", "cldfr")}
    ad, fd, smooth = directional_check(lib, table, x, g)
    assert_mostly_smooth(ad, smooth)
    # aggregate directional derivative over the smooth points
    ad, fd = ad[smooth], fd[smooth]
    assert abs(ad.sum() - fd.sum()) <= 1e-6 * abs(ad).sum(), (ad.sum(), fd.sum())
    # and point by point
    ok = np.abs(ad - fd) <= 1e-6 * np.abs(ad) + 1e-9 * np.abs(ad).max()
    assert ok.mean() > 0.999, f"{(~ok).sum()} of {ok.size} points disagree"


def test_ice_adjust_adjoint_all_outputs_each_field(lib):
    from ice3gb.constants import build_table
    table = build_table(table="phyex")
    x = _state(16 * 16, seed=8, mf=True)
    rng = np.random.default_rng(12)
    g_all = {k: rng.standard_normal(x["th"].shape) for k in OUT}
    for i, k in enumerate(OUT):    # one output at a time, then all together
        ad, fd, smooth = directional_check(lib, table, x, {k: g_all[k]}, seed=i)
        assert_mostly_smooth(ad, smooth, k, share=5e-2)
        ad, fd = ad[smooth], fd[smooth]
        assert abs(ad.sum() - fd.sum()) <= 1e-6 * max(abs(ad).sum(), 1e-300), (k, ad.sum(), fd.sum())
    ad, fd, smooth = directional_check(lib, table, x, g_all)
    assert_mostly_smooth(ad, smooth)
    assert abs(ad[smooth].sum() - fd[smooth].sum()) <= 1e-6 * abs(ad[smooth]).sum()


SRC = ("rcs", "rrs", "ris", "rss", "rgs")
INPR = ("inprc", "inprr", "inpri", "inprs", "inprg")


@pytest.fixture(scope="module")
def sedlib(tmp_path_factory):
    out = tmp_path_factory.mktemp("sed") / "libsed_host.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-I",
                    os.path.join(HERE, "..", "include"), os.path.join(HERE, "sedimentation_host.cpp"), "-o",
                    str(out)], check=True)
    return ctypes.CDLL(str(out))


def _sed_state(nij, seed):
    from ice3gb.state import make_state
    st = {k: v.numpy() for k, v in make_state(nij, 90, seed=seed, precip=True).items()}
    return {"rhodref": st["rho_dry_ref"], "dzz": st["dzz"], "pabs": st["pabs"], "tht": st["th"],
            **{k: st[k] for k in SRC}}


def sed_forward(lib, table, x, fortran):
    nk, nij = x["rhodref"].shape
    c = {k: np.ascontiguousarray(x[k], dtype=np.float64) for k in ("rhodref", "dzz", "pabs", "tht") + SRC}
    out = {k: np.empty((nk, nij)) for k in SRC}
    inpr = {k: np.empty(nij) for k in INPR}
    lib.sed_forward_host(ctypes.byref(table.consts), nij, nk, ctypes.c_double(DT), int(fortran),
                         *[c[k].ctypes.data_as(ctypes.c_void_p) for k in ("rhodref", "dzz", "pabs", "tht")],
                         _ptrs([c[k] for k in SRC]), _ptrs([out[k] for k in SRC]), _ptrs([inpr[k] for k in INPR]))
    return {**out, **inpr}


def sed_vjp(lib, table, x, g, fortran):
    nk, nij = x["rhodref"].shape
    c = {k: np.ascontiguousarray(x[k], dtype=np.float64) for k in ("rhodref", "dzz", "pabs", "tht") + SRC}
    gs = [np.ascontiguousarray(g[k]) if k in g else None for k in SRC]
    gi = [np.ascontiguousarray(g[k]) if k in g else None for k in INPR]
    gx = {k: np.empty((nk, nij)) for k in ("rhodref", "dzz", "pabs", "tht") + SRC}
    scratch = np.empty(5 * nk * nij)
    lib.sed_vjp_host(ctypes.byref(table.consts), nij, nk, ctypes.c_double(DT), int(fortran),
                     *[c[k].ctypes.data_as(ctypes.c_void_p) for k in ("rhodref", "dzz", "pabs", "tht")],
                     _ptrs([c[k] for k in SRC]), _ptrs(gs), _ptrs(gi), _ptrs([gx[k] for k in SRC]),
                     *[gx[k].ctypes.data_as(ctypes.c_void_p) for k in ("rhodref", "dzz", "pabs", "tht")],
                     scratch.ctypes.data_as(ctypes.c_void_p))
    return gx


@pytest.mark.parametrize("fortran", [True, False])
def test_sedimentation_adjoint_matches_finite_differences(sedlib, fortran):
    """Reverse sweep vs centred differences (h = 1e-7, relative directions) of
    <g, (sources after the sweep, surface precipitation)> with N(0,1)
    cotangents, for all nine inputs together and for each alone."""
    from ice3gb.constants import build_table
    table = build_table(table="phyex")
    x = _sed_state(24 * 24, seed=6)
    rng = np.random.default_rng(21)
    g = {k: rng.standard_normal(x["rhodref"].shape) for k in SRC}
    g.update({k: rng.standard_normal(x["rhodref"].shape[1]) for k in INPR})
    # scale the cotangents so that every output contributes at its own size
    y0 = sed_forward(sedlib, table, x, fortran)
    g = {k: v / max(np.abs(y0[k]).max(), 1e-300) for k, v in g.items()}
    gx = sed_vjp(sedlib, table, x, g, fortran)
    h = 1e-7
    for subset in (tuple(gx), *[(k,) for k in gx]):
        dx = {k: (rng.standard_normal(v.shape) * np.abs(v) if k in subset else np.zeros_like(v)) for k, v in x.items()}
        ad = sum(float(np.sum(gx[k] * dx[k])) for k in subset)
        yp = sed_forward(sedlib, table, {k: v + h * dx[k] for k, v in x.items()}, fortran)
        ym = sed_forward(sedlib, table, {k: v - h * dx[k] for k, v in x.items()}, fortran)
        fd = sum(float(np.sum(g[k] * (yp[k] - ym[k]))) for k in g) / (2 * h)
        scale = sum(float(np.sum(np.abs(gx[k] * dx[k]))) for k in subset)
        assert abs(ad - fd) <= 1e-6 * max(scale, 1e-300), (subset, ad, fd)


# ---- against the reference's own derivatives (tests/golden/adjoint_fd.npz) ----

def _reference_fd(g, prefix, h=1e-7):
    jp, j0, jm = (np.asarray(g[f"{prefix}_j{t}"]).ravel() for t in "p0m")
    noise = 4e-16 * (np.abs(j0) + np.abs(jp) + np.abs(jm)) / h
    return (jp - jm) / (2 * h), smooth_points(jp, j0, jm, h), noise


def reference_ice_adjust_check(ad, g):
    """Adjoint directional derivatives against the centred differences of the
    reference IceAdjustJAX: every smooth point within 1e-6."""
    fd, smooth, noise = _reference_fd(g, "ia")
    assert_mostly_smooth(ad, smooth, "ice_adjust vs reference")
    rel = np.abs(ad - fd) / (np.abs(ad) + noise)
    assert rel[smooth].max() <= 1e-6, rel[smooth].max()
    return rel[smooth]


def reference_sedimentation_check(ad, g):
    fd, smooth, noise = _reference_fd(g, "sed")
    assert_mostly_smooth(ad, smooth, "sedimentation vs reference")
    rel = np.abs(ad - fd) / (np.abs(ad) + noise)
    assert rel[smooth].max() <= 1e-6, rel[smooth].max()
    return rel[smooth]


def test_ice_adjust_adjoint_matches_reference_differences(lib):
    """The adjoint (host build) against centred differences of the
    reference's own IceAdjustJAX in FP64 (h = 1e-7, relative directions,
    N(0,1) cotangents on T, rv, rc, ri, cloud fraction; 32 x 90 points)."""
    from conftest import load_golden
    from ice3gb.constants import build_table
    g = load_golden("adjoint_fd")
    table = build_table(table="jax")
    x = {k: g[f"ia_x_{k}"] for k in IN}
    dx = {k: g[f"ia_dx_{k}"] for k in IN}
    gx = vjp(lib, table, x, {k: g[f"ia_g_{k}"] for k in ("t", "rv_out", "rc_out", "ri_out", "cldfr")})
    ad = sum(gx[k].reshape(x[k].shape) * dx[k] for k in IN).ravel()
    reference_ice_adjust_check(ad, g)


def test_sedimentation_adjoint_matches_reference_differences(sedlib):
    """The reverse sweep (host build, the reference JAX semantics) against
    centred differences of the reference's own sedimentation_stat in FP64,
    per column (24 columns x 90 levels)."""
    from conftest import load_golden
    from ice3gb.constants import build_table
    g = load_golden("adjoint_fd")
    table = build_table(table="jax")
    sin = ("rhodref", "dzz", "pabs", "tht") + SRC
    x = {k: g[f"sed_x_{k}"] for k in sin}
    gx = sed_vjp(sedlib, table, x, {k: g[f"sed_g_{k}"] for k in SRC + INPR}, False)
    ad = sum((gx[k] * g[f"sed_dx_{k}"]).sum(axis=0) for k in sin)
    reference_sedimentation_check(ad, g)
