"""OCND2 in ice_adjust (separate liquid and ice clouds, PHYEX
micro/condensation.F90:373-395 and :588-637 with ICECLOUD,
micro/mode_icecloud.F90, and the TIWMX tables, micro/mode_ini_tiwmx.F90).

The reference's JAX ice_adjust has no OCND2 branch (OCND2 = False is fixed
in src/ice3/jax/ice_adjust.py:116) and its Fortran cannot be compiled here,
so the pins are: the oracle's TIWMX tables against the reference's own
e_sat_w / e_sat_i (tests/golden/tiwmx.npz), and the oracle's OCND2 path
against a second, pure-Python restatement of the Fortran on a few hundred
points.  Then the device code's host build (CPU) and the device kernel
(GPU, device and host buffers, with the oracle's conditioning allowance)
against the oracle."""
import ctypes
import math
import os

import numpy as np
import pytest

import test_adjoint_host as H
from conftest import assert_parity, load_golden, rel_err, sensitivity
from helpers import TOL
from test_adjoint_host import lib  # noqa: F401  (host build of the point code, a fixture)

DT = 50.0
EXTRA = ("icldfr", "wcldfr", "ssio", "ssiu", "ifr")


def _table(**kw):
    from ice3gb.constants import build_table
    return build_table(table="jax", overrides={"OCND2": 1.0, **kw})


def _state(nij, seed):
    """Synthetic state with heights (levels from the surface up, first level
    10-300 m above ground) and a per-column ice cloud weight."""
    x = H._state(nij, seed)
    from ice3gb.state import make_state
    dzz = make_state(nij, 90, seed=seed, precip=True)["dzz"].numpy()
    rng = np.random.default_rng(seed + 7)
    z0 = rng.uniform(10.0, 300.0, nij)
    x["zz"] = z0[None, :] + np.concatenate([np.zeros((1, nij)), np.cumsum(dzz[:-1], axis=0)], axis=0)
    x["ice_cld_wgt"] = rng.uniform(0.5, 2.0, nij)
    return x


# ---------------------------------------------------------------------------- pins of the oracle

def test_tiwmx_tables_match_reference_saturation_pressures():
    import oracle
    g = load_golden("tiwmx")
    w, i = oracle.tiwmx_tables(_table())
    j = g["j"].astype(np.int64) - 13200
    np.testing.assert_allclose(w[j], g["esw"], rtol=2e-15, atol=0)
    # ESTABI: the ice formula at and below 273.15 K, the water one above (INI_TIWMX)
    t = g["j"] / 100.0
    np.testing.assert_allclose(i[j], np.where(t > 273.15, g["esw"], g["esi"]), rtol=2e-15, atol=0)
    assert len(w) == 37316 - 13200 + 1


def _ocnd2_point_py(c, x, k, nk, zz_col, wgt, estw, esti, dt):
    """condensation.F90 / ice_adjust.F90 for one point with OCND2 = .TRUE.,
    LSUBG_COND, CB02, written from the Fortran text as plain Python (the JAX
    sources/MF part, ice_adjust.py:268-379, for the rest)."""
    def esat(tab, t):
        jj = int(math.floor(abs(100.0 * t) + 0.5)) * (1 if t >= 0 else -1)   # NINT
        return tab[min(max(jj, 13200), 37316) - 13200]

    t = x["th"] * x["exn"]
    lv = c["LVTT"] + (c["CPV"] - c["CL"]) * (t - c["TT"])
    ls = c["LSTT"] + (c["CPV"] - c["CI"]) * (t - c["TT"])
    cph = c["CPD"] + c["CPV"] * x["rv"] + c["CL"] * (x["rc"] + x["rr"]) + c["CI"] * (x["ri"] + x["rs"] + x["rg"])
    prifact = 0.0
    rt = x["rv"] + x["rc"] + x["ri"] * prifact
    kp = min(k + 1, nk - 1)
    dz = zz_col[kp] - zz_col[kp - 1]
    # ICECLOUD(PP, PZ, PDZ, PT, PR=rv, PTSTEP=1, PPBLH=-1, PWCLD=-1, XW2D=10)
    p, z = x["pabs"], zz_col[k]
    zr = max(0.0, x["rv"] * 1.0)
    sifrc = 0.0
    za = zr * p / (c["EPSILO"] + zr)
    rhw = za / esat(estw, t)
    rhi = za / esat(esti, t)
    i2w = esat(estw, t) / esat(esti, t)
    ssiu = min(i2w, rhi)
    ssio = ssiu
    if t > 273.1 or zr <= 0.0 or esat(esti, t) >= p * 0.5:
        ssiu = ssiu - 1.0
        ssio = ssiu
    else:
        rhin = max(0.05, min(1.0, rhw))
        drhdz = rhin * c["GRAVITY0"] / (t * c["RD"]) * (c["EPSILO"] * c["LVTT"] / (c["CPD"] * t) - 1.0)
        zzf = min(1.0, max(0.0, z * 0.001))
        rhdist = math.sqrt(2500.0 * 3.0e-4 ** 2 + 2500.0 * 3.0e-4 ** 2 + (1.0 - zzf) * (dz * drhdz) ** 2
                           + zzf * dz * 1.0e-2 ** 2)
        if zzf > 0.1:
            rhdist = rhdist / (1.0 + rhdist)
        rhlim = max(0.5, min(0.99, 1.0 - 0.5 * rhdist))
        rhdif = (1.0 - rhw) / (1.0 - rhlim)
        rhdif = 1.0 - math.sqrt(max(0.0, rhdif))
        wcld = min(1.0, max(rhdif, 0.0))
        sifrc = wcld
        rhlimice = 1.0 + i2w * (rhlim - 1.0)
        if rhlim <= 0.999:
            rhdif = (rhi - rhlimice) * (1.0 / (1.0 - rhlimice))
            if wcld == 0.0:
                sifrc = min(1.0, 0.5 * max(0.0, rhdif))
            else:
                sifrc = min(1.0, (1.0 - 1.0 / i2w) * 0.5 / (1.0 - rhlim))
                sifrc = min(1.0, wcld + sifrc)
        if sifrc > 0.01:
            ssiu = sifrc + rhlimice * (1.0 - sifrc)
            ssio = (rhi - (1.0 - sifrc) * ssiu) / sifrc
        else:
            sifrc = 0.0
            ssiu = max(0.0, sifrc + rhlimice * (1.0 - sifrc) + 2.0 * min(0.0, rhi - rhlimice))
        ssio = min(i2w, ssio) - 1.0
        ssiu = max(0.0, ssiu) - 1.0
    icldfr = sifrc
    pv = min(esat(estw, t), 0.99 * p)
    piv = min(esat(esti, t), 0.99 * p)
    frac = 0.0
    qsl = c["RD"] / c["RV"] * pv / (p - pv)
    qsi = c["RD"] / c["RV"] * piv / (p - piv)
    qsl = (1.0 - frac) * qsl + frac * qsi
    lvs = (1.0 - frac) * lv + frac * ls
    ah = lvs * qsl / (c["RV"] * t ** 2) * (c["RV"] * qsl / c["RD"] + 1.0)
    a = 1.0 / (1.0 + lvs / cph * ah)
    sbar = a * (rt - qsl + ah * lvs * (x["rc"] + x["ri"] * prifact) / cph)
    sq = x["sigqsat"]
    sigma = math.sqrt((2 * x["sigs"]) ** 2 + (sq * qsl * a) ** 2) if sq != 0.0 else 2 * x["sigs"]
    sigma = max(1e-10, sigma)
    q1 = sbar / sigma
    if 0.0 < q1 <= 2.0:
        cond = min(math.exp(-1.0) + 0.66 * q1 + 0.086 * q1 ** 2, 2.0)
    elif q1 > 2.0:
        cond = q1
    else:
        cond = math.exp(1.2 * q1 - 1.0)
    cond *= sigma
    cldfr = 0.0 if cond < 1e-12 else max(0.0, min(1.0, 0.5 + 0.36 * math.atan(1.55 * q1)))
    if cldfr == 0.0:
        cond = 0.0
    rc_out = (1.0 - frac) * cond
    lwinc = rc_out - x["rc"]
    if abs(lwinc) > 1.0e-12 and esat(estw, t) < p * 0.5:
        rcold = rc_out
        rc_out = cond - 0.0          # ZRSDIF = 0: PRV_IN < ZRSW = -9999 never holds
    else:
        rcold = x["rc"]
    wcldfr = cldfr
    dum1 = min(1.0, 20.0 * rc_out * math.sqrt(dz) / qsl)
    dum3 = max(0.0, icldfr - wcldfr)
    dum4 = x["ri"] if k == 0 else x["ri"] + x["rs"] * 0.5 + x["rg"] * 0.25
    dum4 = max(0.0, min(1.0, wgt * dum4 * math.sqrt(dz) / qsi))
    dum2 = (0.8 * cldfr + 0.2) * min(1.0, dum1 + dum4 * cldfr)
    cldfr = min(1.0, dum2 + (0.5 * dum3 + 0.5) * dum4)
    ri_out = x["ri"]
    t = t + ((rc_out - rcold) * lv + (ri_out - x["ri"]) * ls) / cph
    rv_out = rt - rc_out - ri_out * prifact
    # sources (ice_adjust.py:268-281) and the mass-flux part (:284-305, cf_mf = 0 here)
    w1 = (rc_out - x["rc"]) / dt
    w1 = max(w1, -x["rcs"]) if w1 < 0 else min(w1, x["rvs"])
    rvs, rcs = x["rvs"] - w1, x["rcs"] + w1
    ths = x["ths"] + w1 * lv / (cph * x["exn_ref"])
    cldfr = min(1.0, cldfr + x["cf_mf"])
    return dict(t=t, rv_out=rv_out, rc_out=rc_out, ri_out=ri_out, cldfr=cldfr, rvs=rvs, rcs=rcs, ths=ths,
                icldfr=icldfr, wcldfr=wcldfr, ssio=ssio, ssiu=ssiu)


def test_oracle_matches_python_restatement_of_the_fortran():
    import oracle
    t = _table()
    x = _state(12 * 12, seed=3)
    ref = oracle.ice_adjust(t, x, DT)
    estw, esti = oracle.tiwmx_tables(t)
    nk, nij = x["th"].shape
    rng = np.random.default_rng(0)
    pts = [(k, j) for k, j in zip(rng.integers(0, nk, 400), rng.integers(0, nij, 400))]
    pts += [(0, 3), (nk - 1, 5), (nk - 2, 7)]       # bottom (no snow/graupel term), top (thickness below)
    seen_cloud = seen_ice = 0
    for k, j in pts:
        xp = {key: (x[key][k, j] if x[key].ndim == 2 else x[key][j]) for key in H.IN}
        got = _ocnd2_point_py(t.values, xp, k, nk, x["zz"][:, j], x["ice_cld_wgt"][j], estw, esti, DT)
        for key, v in got.items():
            r = ref[key][k, j]
            assert abs(v - r) <= 1e-12 * max(abs(r), 1e-300) + 1e-300, (key, k, j, v, r)
        seen_cloud += got["wcldfr"] > 0
        seen_ice += got["icldfr"] > 0
    assert seen_cloud > 20 and seen_ice > 20


# ---------------------------------------------------------------------------- host build and properties

def _host_ocnd2(lib, t, x):  # noqa: F811
    import oracle
    estw, esti = oracle.tiwmx_tables(t)
    tab = np.concatenate([estw, esti])
    nk, nij = x["th"].shape
    ins = [np.ascontiguousarray(x[k], dtype=np.float64).ravel() for k in H.IN]
    out = [np.empty(nk * nij) for _ in H.OUT]
    out2 = [np.empty(nk * nij) for _ in range(4)]
    lib.ia_ocnd2_host(ctypes.byref(t.consts), ctypes.c_double(DT), ctypes.c_long(nij), ctypes.c_long(nk),
                      H._ptrs(ins), np.ascontiguousarray(x["zz"]).ctypes.data_as(ctypes.c_void_p),
                      np.ascontiguousarray(x["ice_cld_wgt"]).ctypes.data_as(ctypes.c_void_p),
                      tab.ctypes.data_as(ctypes.c_void_p), H._ptrs(out), H._ptrs(out2))
    res = {k: v.reshape(nk, nij) for k, v in zip(H.OUT, out)}
    res.update({k: v.reshape(nk, nij) for k, v in zip(EXTRA[:4], out2)})
    return res


@pytest.mark.parametrize("sigqsat", [0.02, 0.0])
def test_host_build_matches_oracle(lib, sigqsat):  # noqa: F811
    import oracle
    t = _table()
    x = _state(32 * 32, seed=11)
    x["sigqsat"] = np.full_like(x["sigqsat"], sigqsat)
    ref = oracle.ice_adjust(t, x, DT)
    got = _host_ocnd2(lib, t, x)
    for k in H.OUT + EXTRA[:4]:
        assert rel_err(got[k], ref[k]) <= TOL, k
    np.testing.assert_array_equal(ref["ifr"], 10.0)


def test_ocnd2_properties():
    """Ice is left to the microphysics (ri_out = ri, no ice source), the
    adjustment only exchanges vapour and liquid, and the fractions stay in
    [0, 1]."""
    import oracle
    x = _state(32 * 32, seed=12)
    ref = oracle.ice_adjust(_table(), x, DT)
    np.testing.assert_array_equal(ref["ri_out"], x["ri"])
    np.testing.assert_array_equal(ref["ris"], x["ris"])
    tot_in = x["rv"] + x["rc"]
    assert np.abs(ref["rv_out"] + ref["rc_out"] - tot_in).max() <= 1e-15 * np.abs(tot_in).max()
    for k in ("icldfr", "wcldfr", "cldfr"):
        assert ref[k].min() >= 0.0 and ref[k].max() <= 1.0, k
    assert (ref["icldfr"] > 0).sum() > 100 and (ref["wcldfr"] > 0).sum() > 100
    # the radiative cloud fraction differs from the water cloud fraction where ice is present
    assert np.count_nonzero(ref["cldfr"] != ref["wcldfr"]) > 100


def test_ocnd2_needs_subgrid_condensation_and_heights():
    import oracle
    x = _state(8 * 8, seed=13)
    with pytest.raises(RuntimeError):
        oracle.ice_adjust(_table(LSUBG_COND=0.0), x, DT)


# ---------------------------------------------------------------------------- GPU

@pytest.mark.gpu
@pytest.mark.parametrize("buffers", ["device", "host"])
def test_device_matches_oracle(buffers):
    import oracle
    import torch
    from ice3gb import IceAdjust
    x = _state(64 * 64, seed=21)
    ia = IceAdjust()
    ia.table = _table()
    # the sources are differences of nearly equal terms at some points: the
    # oracle's own spread under 1e-13 input perturbations bounds those
    ref, spread = sensitivity(lambda y: oracle.ice_adjust(ia.table, y, DT, srcs=True), x)
    names = H.IN
    if buffers == "device":
        dev = {k: torch.as_tensor(v).cuda() for k, v in x.items()}
        res = ia(**{k: dev[k] for k in names}, timestep=DT, return_srcs=True, zz=dev["zz"],
                 ice_cld_wgt=dev["ice_cld_wgt"])
        res = [r.cpu().numpy() for r in res]
    else:
        res = ia(**{k: x[k] for k in names}, timestep=DT, return_srcs=True, zz=x["zz"],
                 ice_cld_wgt=x["ice_cld_wgt"])
    assert len(res) == 16 + 1 + 5
    order = ("t", "rv_out", "rc_out", "ri_out", "cldfr", "hlc_hrc", "hlc_hcf", "hli_hri", "hli_hcf", "cph", "lv", "ls",
             "rvs", "rcs", "ris", "ths", "srcs") + EXTRA
    for k, v in zip(order, res):
        assert_parity(v, ref[k], spread[k], k)
    assert ia.handle.status() == 0


@pytest.mark.gpu
def test_device_rejects_ocnd2_without_levels():
    import torch
    from ice3gb import IceAdjust, _abi
    x = _state(8 * 8, seed=22)
    ia = IceAdjust()
    ia.table = _table()
    dev = {k: torch.as_tensor(np.ascontiguousarray(v[:1] if v.ndim == 2 and k != "ice_cld_wgt" else v)).cuda()
           for k, v in x.items()}
    with pytest.raises(_abi.Ice3gbError, match="nk >= 2"):
        ia(**{k: dev[k] for k in H.IN}, timestep=DT, zz=dev["zz"], ice_cld_wgt=dev["ice_cld_wgt"])
    with pytest.raises(ValueError, match="zz"):
        ia(**{k: dev[k] for k in H.IN}, timestep=DT)


# ---------------------------------------------------------------------------- OCND2 in rain_ice: pins

def _tiwmx_fun(v, tt):
    """The TIWMX table entry at NINT(100 T) (mode_tiwmx.F90) of the functions of
    mode_tiwmx_fun.F90 as INI_TIWMX fills them."""
    j = min(max(int(math.floor(abs(100.0 * tt) + 0.5)), 13200), 37316)
    T = j / 100.0
    TT = v["TT"]
    esw = math.exp(v["ALPW"] - v["BETAW"] / T - v["GAMW"] * math.log(T))
    esi_f = esw if T >= TT else math.exp(v["ALPI"] - v["BETAI"] / T - v["GAMI"] * math.log(T))   # ESATI, SIGN(0.5, 0) = 0.5
    estabi = esw if T > 273.15 else esi_f
    a2 = (v["LSTT"] + (v["CPV"] - v["CI"]) * (T - TT)) ** 2 / (2.38E-2 + 0.0071E-2 * (T - TT)) / (T ** 2 * v["RV"])
    bb3 = v["RV"] / (0.211E-4 * (T / TT) ** 1.94 * v["P00"]) * T / esi_f
    am3 = 0.0 if T > 273.15 else 1000. * math.exp(12.96 * (esw / esi_f - 1.) - 0.639)
    zzt = max(0., min(1., (TT - T) / 20.))
    redin = 1. - (1. - zzt) / (zzt ** 3 + (1. - zzt) ** 3) ** .333
    return dict(esi=estabi, a2=a2, bb3=bb3, am3=am3, redin=redin)


def ocnd2_rates_py(v, x):
    """ICE4_NUCLEATION's OCND2 branch (ice4_nucleation.func.h:127-136), the
    tabulated derived fields and collision factors (mode_ice4_tendencies.F90:
    303-346, LLTAB, LLCOL) and ICE4_FAST_RI_RS (mode_ice4_fast_ri_rs.F90,
    LMODICEDEP = .FALSE.) for one point, written from the Fortran text."""
    t, rho, p, rv, rc, rr, ri, rs, rg, cit, ssio, ssiu, ifr, icldfr, zzz, conc = x
    TT = v["TT"]
    if t < TT and rv > v["V_RTMIN"]:
        zzw = _tiwmx_fun(v, t)["redin"] * max(0.1, ((20000. - min(20000., zzz)) / 20000.) ** 4) \
            * _tiwmx_fun(v, max(v["FRMIN27"], t))["am3"] * (0.0001 + 0.9999 * icldfr)
        zzw = min(zzw, 50.E3)
        cit = max(zzw + cit, cit)
    tab = _tiwmx_fun(v, t)
    esi = tab["esi"]
    ssi = rv * (p - esi) / (v["EPSILO"] * esi) - 1.0
    ai = tab["a2"] + tab["bb3"] * p
    zconc = conc * 0.000001
    colf = acrf = 0.00001
    if rc > 1.0E-10:
        rcw = 0.1 * (0.75 * rc * rho / (v["PI"] * zconc)) ** 0.333
        vt = 1.19E6 * rcw ** 2 if rcw < 0.0065 else 8000. * rcw
        vt = min(10., vt)
        st = max(0.01, 2. * (100. - vt) * vt / (v["GRAVITY0"] * 10.))
        if st > 0.1:
            colf = max(0.01, min(1., 0.939 * st ** 2.657))
        if rr > 1.0E-10 and rcw > 1.0E-5:
            r20 = math.exp(rcw * 2000.)
            acrf = (r20 - 1.) / (r20 + 1.)
    timesc, dicrit = v["FRMIN14"], v["FRMIN15"]
    rilars = 0.
    if ri > 0.0 and ssi > 0.001:
        rilars = min(ri, ri / (87.5 * dicrit ** 2 * ai / ssi))
    rvdepi = 0.
    w2d = 1. / (ifr * icldfr + 1. - icldfr)
    if (p * 0.5 - esi) > 0. and cit > 0.:
        xw2d13 = ifr ** 0.333
        wcitred23 = 0.1 ** 0.667
        tc = max(-18., min(-1., t - TT))
        hu = min(0.15, max(0., ssi))
        cryssha = 1.1 + 3. * hu * (1. + math.sin(0.64 * tc - 1.3))
        qimax = 366.5 * dicrit ** 3 * cit * 0.1 / rho
        ci2s = 0.
        if ri > 1.0e-12 and timesc > 0.:
            ci2s = ri * (1. - min(1., 0.5 * qimax / ri)) * (1. - icldfr) * w2d / (timesc * 0.5)
        zzwc = cryssha * 0.878 / ai * (cit / rho) ** 0.667 * (max(v["I_RTMIN"], ri) * w2d) ** 0.333
        if ssio > 0. and icldfr > 0.02:
            rvdepi += zzwc * xw2d13 * ssio * icldfr
        if ssiu < 0. and icldfr < 0.98:
            rilars += ci2s
            rvdepi += zzwc * wcitred23 * ssiu * (1. - icldfr)
    return [cit, esi, ssi, ai, colf, acrf, rilars, rvdepi]


def test_oracle_ocnd2_rain_ice_pieces_match_python_restatement():
    import oracle
    from ice3gb.constants import build_table
    t = build_table(table="phyex", overrides={"OCND2": 1.0})
    v = {k: float(x) for k, x in t.values.items()}
    rng = np.random.default_rng(9)
    n = 500
    T = rng.uniform(225.0, 285.0, n)
    rho = rng.uniform(0.3, 1.2, n)
    p = rho * 287.0 * T
    mix = lambda pz: np.exp(rng.uniform(np.log(1e-9), np.log(3e-3), n)) * (rng.uniform(size=n) > pz)  # noqa: E731
    rv = rng.uniform(0.5, 1.2, n) * 0.622 * 611.0 * np.exp(17.5 * (T - 273.15) / (T - 36.0)) / p
    x = np.stack([T, rho, p, rv, mix(0.3), mix(0.3), mix(0.3), mix(0.3), mix(0.3),
                  rng.uniform(0, 2e4, n) * (rng.uniform(size=n) > 0.3),        # cit
                  rng.uniform(-0.3, 0.2, n), rng.uniform(-0.5, 0.0, n), np.full(n, 10.0),   # ssio, ssiu, ifr
                  rng.uniform(0, 1, n) * (rng.uniform(size=n) > 0.2),          # icldfr
                  rng.uniform(0, 25000.0, n), rng.choice([1e8, 3e8, 5e8], n)], axis=1)   # zzz, conc
    out = np.empty((n, 8))
    lib = oracle.load()
    lib.ice3o_ocnd2_rates(ctypes.byref(t.consts), ctypes.c_long(n), np.ascontiguousarray(x).ctypes.data_as(
        ctypes.c_void_p), out.ctypes.data_as(ctypes.c_void_p))
    active = np.zeros(8, dtype=int)
    for i in range(n):
        ref = np.array(ocnd2_rates_py(v, tuple(x[i])))
        np.testing.assert_allclose(out[i], ref, rtol=1e-12, atol=1e-300, err_msg=f"point {i}")
        active += (ref != 0.0) & (ref != x[i, 9])
    assert np.all(active[[0, 4, 5, 6, 7]] > 10), active


# ---------------------------------------------------------------------------- OCND2 in rain_ice: host build, device

def ocnd2_rain_ice_state(nij, seed):
    """A rain_ice state (ABI names) with the OCND2 ice_adjust outputs of the
    same atmosphere (ssio, ssiu, ifr, icldfr)."""
    import oracle
    from ice3gb.constants import build_table
    from ice3gb.state import make_state
    from test_gpu_rain_ice import _abi_rain_ice_state
    st = {k: v.numpy() for k, v in make_state(nij, 90, seed=seed, precip=True).items()}
    x = _abi_rain_ice_state(st)
    ia = _state(nij, seed)
    oa = oracle.ice_adjust(build_table(table="jax", overrides={"OCND2": 1.0}), ia, DT)
    for k in ("ssio", "ssiu", "ifr", "icldfr"):
        x[k] = oa[k]
    return x


def _ri_table(**kw):
    from ice3gb.constants import build_table
    return build_table(table="phyex", overrides={"OCND2": 1.0, **kw})


RI_OUT = ("ths", "rvs", "rcs", "rrs", "ris", "rss", "rgs", "cit", "inprc", "inprr", "inpri", "inprs", "inprg")


def _ri_scale(x, ref, fl, k):
    rhodz = x["rhodref"] * x["dzz"]
    s = np.abs(x[k]) + np.abs(ref[k])
    key = {"rcs": "c", "rrs": "r", "ris": "i", "rss": "s", "rgs": "g"}.get(k)
    if key:
        f_ = fl["fpr_" + key]
        fa = np.concatenate([f_[1:], np.zeros_like(f_[:1])], axis=0)
        s = s + (np.abs(f_) + np.abs(fa)) / rhodz
    return s


@pytest.mark.parametrize("kw", [{}, {"SUBG_RC_RR_ACCR": 1.0, "SUBG_RR_EVAP": 2.0}, {"SUBG_RR_EVAP": 1.0},
                                {"SUBG_RR_EVAP": 1.0, "MRSTEP": 5e-5}])
def test_ocnd2_rain_ice_host_build_matches_oracle(kw):
    import oracle
    import subprocess
    from ice3gb import _abi
    from test_hail import _report_ties, _untie
    d = os.path.dirname(os.path.abspath(__file__))
    libs = {}
    for name in ("rain_ice_point_host", "sedimentation_host"):
        out = f"/tmp/ocnd2_{name}_{os.getpid()}.so"
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-I",
                        os.path.join(d, "..", "include"), os.path.join(d, f"{name}.cpp"), "-o", out], check=True)
        libs[name] = ctypes.CDLL(out)
    t = _ri_table(LSEDIM_AFTER=1.0, LDEPOSC=0.0, **kw)
    nij, nk = 24 * 24, 90
    x = ocnd2_rain_ice_state(nij, seed=3)
    keep, f = {}, _abi.RainIceFields()
    for k in ("exn", "dzz", "rhodref", "exnref", "pabs", "cldfr", "sigs", "tht", "rvt", "rct", "rrt", "rit", "rst",
              "rgt", "sea", "town", "ssio", "ssiu", "ifr", "icldfr"):
        keep[k] = np.ascontiguousarray(x[k], dtype=np.float64)
        setattr(f, k, keep[k].ctypes.data)
    for k in ("cit", "hlc_hrc", "hlc_hcf", "hli_hri", "hli_hcf", "ths", "rvs", "rcs", "rrs", "ris", "rss", "rgs"):
        keep[k] = np.array(x[k], dtype=np.float64)
        setattr(f, k, keep[k].ctypes.data)
    for k in ("evap3d", "rainfr"):
        keep[k] = np.zeros((nk, nij))
        setattr(f, k, keep[k].ctypes.data)
    for k in ("inprc", "inprr", "inpri", "inprs", "inprg"):
        keep[k] = np.zeros(nij)
        setattr(f, k, keep[k].ctypes.data)
    lib = oracle.load()
    tw = np.empty(6 * 24117)
    lib.ice3o_tiwmx_all(ctypes.byref(t.consts), tw.ctypes.data_as(ctypes.c_void_p))
    keys = np.zeros(nij * nk, dtype=np.uint32)
    capped = libs["rain_ice_point_host"].rain_ice_points_host_ocnd2(
        ctypes.byref(t.consts), ctypes.byref(t.luts), nij, nk, ctypes.c_double(DT), 256, ctypes.byref(f),
        tw.ctypes.data_as(ctypes.c_void_p), keys.ctypes.data_as(ctypes.c_void_p))
    assert capped == 0
    libs["sedimentation_host"].sed_stat_rain_ice_host(ctypes.byref(t.consts), nij, nk, ctypes.c_double(DT),
                                                      ctypes.byref(f))
    ref, spread = sensitivity(lambda y: oracle.rain_ice(t, y, DT)[0], x, rel=1e-12, trials=4)
    fl, _ = oracle.rain_ice(t, x, DT, with_fpr=True, with_ties=True)
    spread, share, exempt = _untie(spread, fl["tie"])
    for k in RI_OUT:
        sc = _ri_scale(x, ref, fl, k) if k not in ("cit",) and not k.startswith("inpr") else None
        stats = assert_parity(keep[k], ref[k], spread[k], f"ocnd2 host/{k}", scale=sc, max_frac_conditioned=0.01 + share[k])
        _report_ties(f"ocnd2 host/{k}", keep[k], ref[k], sc, exempt[k], stats)


@pytest.mark.parametrize("sedim", [1.0, 0.0])
def test_ocnd2_rain_ice_water_budget(sedim):
    import oracle
    t = _ri_table(SEDIM=sedim)
    nij, nk = 16 * 16, 90
    x = ocnd2_rain_ice_state(nij, seed=4)
    out, bits = oracle.rain_ice(t, x, DT)
    assert bits == 0
    rhodz = x["rhodref"] * x["dzz"]
    src = ("rvs", "rcs", "rrs", "ris", "rss", "rgs")
    d = sum(out[k] - x[k] for k in src)
    col = (rhodz * d).sum(axis=0) * DT
    precip = sum(out[k] for k in ("inprc", "inprr", "inpri", "inprs", "inprg")) * t.values["RHOLW"] * DT
    scale = (rhodz * sum(np.abs(x[k]) for k in src)).sum(axis=0) * DT
    assert np.abs(col + precip).max() <= 1e-12 * scale.max()


@pytest.mark.gpu
@pytest.mark.parametrize("after", [False, True])
def test_ocnd2_rain_ice_device_matches_oracle(after):
    import oracle
    import torch
    from ice3gb import RainIce
    from test_hail import _report_ties, _untie
    t = _ri_table()
    nij = 32 * 32
    x = ocnd2_rain_ice_state(nij, seed=5)
    ref, spread = sensitivity(lambda y: oracle.rain_ice(t, y, DT, lsedim_after=int(after))[0], x, rel=1e-12,
                              trials=4)
    fl, _ = oracle.rain_ice(t, x, DT, lsedim_after=int(after), with_fpr=True, with_ties=True)
    spread, share, exempt = _untie(spread, fl["tie"])
    ri = RainIce()
    ri.table = t
    m = {"exn": "exn", "dzz": "dzz", "rhodref": "rhodref", "exnref": "exnref", "pres": "pabs", "cldfr": "cldfr",
         "sigs": "sigs", "th_t": "tht", "rv_t": "rvt", "rc_t": "rct", "rr_t": "rrt", "ri_t": "rit", "rs_t": "rst",
         "rg_t": "rgt", "ci_t": "cit", "hlc_hrc": "hlc_hrc", "hlc_hcf": "hlc_hcf", "hli_hri": "hli_hri",
         "hli_hcf": "hli_hcf", "ths": "ths", "rvs": "rvs", "rcs": "rcs", "rrs": "rrs", "ris": "ris", "rss": "rss",
         "rgs": "rgs", "sea": "sea", "town": "town", "ssio": "ssio", "ssiu": "ssiu", "ifr": "ifr", "icldfr": "icldfr"}
    state = {k: torch.as_tensor(np.ascontiguousarray(x[v])).cuda() for k, v in m.items()}
    new, diag = ri(state, DT, lsedim_after=after)
    got = {"cit": new["ci_t"].cpu().numpy()}
    for k in ("ths", "rvs", "rcs", "rrs", "ris", "rss", "rgs"):
        got[k] = new[k].cpu().numpy()
    for k in ("inprc", "inprr", "inpri", "inprs", "inprg"):
        got[k] = diag[k].cpu().numpy()
    for k in RI_OUT:
        sc = _ri_scale(x, ref, fl, k) if k not in ("cit",) and not k.startswith("inpr") else None
        stats = assert_parity(got[k], ref[k], spread[k], f"ocnd2 device/{k}", scale=sc, max_frac_conditioned=0.01 + share[k])
        _report_ties(f"ocnd2 device/{k}", got[k], ref[k], sc, exempt[k], stats)
    assert ri.device_status() == 0


@pytest.mark.gpu
@pytest.mark.parametrize("kw", [{"SUBG_RC_RR_ACCR": 1.0, "SUBG_RR_EVAP": 2.0}, {"SUBG_RR_EVAP": 1.0}])
def test_ocnd2_rain_ice_warm_options_device_matches_oracle(kw):
    """OCND2 with the subgrid warm-process options (the OCND2 branches leave
    ICE4_WARM and ICE4_COMPUTE_PDF as they are)."""
    import oracle
    from test_hail import _report_ties, _untie
    from test_time_splitting import _ocnd2_device
    t = _ri_table(**kw)
    x = ocnd2_rain_ice_state(32 * 32, seed=6)
    ref, spread = sensitivity(lambda y: oracle.rain_ice(t, y, DT)[0], x, rel=1e-12, trials=4)
    fl, _ = oracle.rain_ice(t, x, DT, with_fpr=True, with_ties=True)
    spread, share, exempt = _untie(spread, fl["tie"], sed_after=False)
    got, ri = _ocnd2_device(t, x)
    for k in RI_OUT:
        sc = _ri_scale(x, ref, fl, k) if k not in ("cit",) and not k.startswith("inpr") else None
        stats = assert_parity(got[k], ref[k], spread[k], f"ocnd2 warm {kw}/{k}", scale=sc, max_frac_conditioned=0.01 + share[k])
        _report_ties(f"ocnd2 warm {kw}/{k}", got[k], ref[k], sc, exempt[k], stats)
    assert ri.device_status() == 0
