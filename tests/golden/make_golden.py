"""Generate the golden vectors in tests/golden/*.npz from the reference code.

Runs maurinl26/dwarf-p-ice3's own JAX implementation, unmodified, in float64
through the numpy stand-in of refshim.py:

* ``IceAdjustJAX.__call__``            (src/ice3/jax/ice_adjust.py:139), also on the
  states of the reference's own tests (tests/components/test_ice_adjust_jax.py)
* ``sedimentation_stat``               (src/ice3/jax/stencils/sedimentation.py:58)
* the ICE4 process stencils            (src/ice3/jax/stencils/ice4_*.py), hard pass
* ``ice4_derived_fields`` / ``ice4_slope_parameters`` (stencils/ice4_tendencies.py:191,248)
* ``ice4_rainfr_vert``                 (stencils/rain_ice.py:272)
* ``ice4_warm`` with the CLFR / PRFR evaporation options (stencils/ice4_warm.py:15)
* the SRC_1D table                     (phyex_common/lookup_table.py:4)
* ``e_sat_w`` / ``e_sat_i`` on the TIWMX grid (jax/functions/tiwmx.py:18,60)
* centred differences of ``IceAdjustJAX`` and ``sedimentation_stat`` for the
  adjoint checks
* the RAIN_ICE / ICE4_STEPPING stencils: ``rain_ice_thermo``, ``rain_ice_mask``,
  ``rain_ice_total_tendencies``, ``fog_deposition`` (stencils/rain_ice.py),
  ``ice4_total_tendencies_update`` (stencils/ice4_tendencies.py:330),
  ``ice4_step_limiter``, ``state_update`` (stencils/ice4_stepping.py:109,232),
  ``ice4_correct_negativities`` (stencils/ice4_correct_negativities.py:14)

Inputs are seeded synthetic states (ice3gb.state.make_state) and seeded
random point sets; both inputs and reference outputs are stored.

Usage:  python tests/golden/make_golden.py [--reference-src DIR]
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "dwarf-p-ice3_gb300"))
sys.path.insert(0, HERE)

DT = 50.0


def _shim(a):
    import refshim
    return np.asarray(a, dtype=np.float64).view(refshim.ShimArray)


def _np(st):
    return {k: v.numpy().copy() for k, v in st.items()}


def ice_adjust_cases(IceAdjustJAX, Phyex):
    from ice3gb.state import make_state

    ia = IceAdjustJAX(Phyex("AROME", TSTEP=DT), jit=False)
    cases = {}
    # config-0 distribution (AROME, CB02, sigqsat = 0.02), 32 columns x 90 levels
    st = _np(make_state(32, 90, seed=0))
    cases["ia_std"] = st
    # mass-flux and source terms active, varying sigqsat (incl. zeros), NRR=6
    st2 = _np(make_state(24, 90, seed=1, precip=True))
    rng = np.random.default_rng(11)
    shape = st2["pabs"].shape
    st2["sigqsat"] = np.where(rng.random(shape) < 0.2, 0.0, rng.uniform(0.0, 0.05, shape))
    st2["cf_mf"] = np.where(rng.random(shape) < 0.5, rng.uniform(0, 1, shape), 0.0)
    st2["rc_mf"] = np.where(rng.random(shape) < 0.5, 10 ** rng.uniform(-8, -3, shape), 0.0)
    st2["ri_mf"] = np.where(rng.random(shape) < 0.5, 10 ** rng.uniform(-8, -3, shape), 0.0)
    st2["rvs"] = rng.uniform(-1e-6, 1e-5, shape)
    st2["rcs"] = rng.uniform(-1e-7, 1e-6, shape)
    st2["ris"] = rng.uniform(-1e-7, 1e-6, shape)
    st2["ths"] = rng.uniform(-1e-3, 1e-3, shape)
    cases["ia_mf"] = st2
    out = {}
    names = ("t", "rv_out", "rc_out", "ri_out", "cldfr", "hlc_hrc", "hlc_hcf", "hli_hri", "hli_hcf", "cph", "lv",
             "ls", "rvs", "rcs", "ris", "ths")
    for cname, st in cases.items():
        nk, nij = st["pabs"].shape
        sigq = st["sigqsat"] if st["sigqsat"].ndim == 2 else np.broadcast_to(st["sigqsat"], (nk, nij)).copy()
        res = ia(sigqsat=sigq, pabs=st["pabs"], sigs=st["sigs"], th=st["th"], exn=st["exn"],
                 exn_ref=st["exn_ref"], rho_dry_ref=st["rho_dry_ref"], rv=st["rv"], rc=st["rc"], ri=st["ri"],
                 rr=st["rr"], rs=st["rs"], rg=st["rg"], cf_mf=st["cf_mf"], rc_mf=st["rc_mf"],
                 ri_mf=st["ri_mf"], rvs=st["rvs"], rcs=st["rcs"], ris=st["ris"], ths=st["ths"], timestep=DT)
        rec = {f"in_{k}": np.asarray(v) for k, v in st.items() if k in (
            "sigqsat", "pabs", "sigs", "th", "exn", "exn_ref", "rho_dry_ref", "rv", "rc", "ri", "rr", "rs",
            "rg", "cf_mf", "rc_mf", "ri_mf", "rvs", "rcs", "ris", "ths")}
        rec.update({f"out_{n}": np.asarray(r, dtype=np.float64) for n, r in zip(names, res)})
        out[cname] = rec
    return out


def sedimentation_case(sedimentation_stat, Phyex):
    from ice3gb.state import make_state

    ext = dict(Phyex("AROME", TSTEP=DT).to_externals())
    ext.update(LBC_LAND=ext["LBC_1"], LBC_SEA=ext["LBC_2"], FSEDC_LAND=ext["FSEDC_1"], FSEDC_SEA=ext["FSEDC_2"])
    st = _np(make_state(24, 90, seed=2, precip=True))
    rng = np.random.default_rng(22)
    nk, nij = st["pabs"].shape
    # sources = mixing ratio / dt with a few negative sources
    src = {}
    for k, r in (("rcs", "rc"), ("rrs", "rr"), ("ris", "ri"), ("rss", "rs"), ("rgs", "rg")):
        src[k] = st[r] / DT
    src["ris"] = np.where(rng.random((nk, nij)) < 0.3, 10 ** rng.uniform(-8, -4, (nk, nij)) / DT, src["ris"])
    src["rcs"][0, :3] = -1e-9
    sea = rng.uniform(0, 1, nij)
    town = rng.uniform(0, 0.5, nij)
    T = lambda a: np.ascontiguousarray(a.T[None, :, :])
    res = sedimentation_stat(T(st["rho_dry_ref"]), T(st["dzz"]), T(st["pabs"]), T(st["th"]), T(src["rcs"]),
                             T(src["rrs"]), T(src["ris"]), T(src["rss"]), T(src["rgs"]), sea[None, :, None],
                             town[None, :, None], ext)
    names = ("rcs", "rrs", "ris", "rss", "rgs", "fpr_c", "fpr_r", "fpr_i", "fpr_s", "fpr_g", "inprc", "inprr",
             "inpri", "inprs", "inprg")
    rec = {"in_rhodref": st["rho_dry_ref"], "in_dzz": st["dzz"], "in_pabs": st["pabs"], "in_tht": st["th"],
           "in_sea": sea, "in_town": town}
    rec.update({f"in_{k}": v for k, v in src.items()})
    for n, r in zip(names, res):
        r = np.asarray(r, dtype=np.float64)
        rec[f"out_{n}"] = r[0].T.copy() if r.ndim == 3 else r[0].copy()
    return {"sed_jax": rec}


def process_cases(mods, Phyex):
    """Hard-pass ICE4 processes on seeded random points."""
    ext = dict(Phyex("AROME", TSTEP=DT).to_externals())
    rng = np.random.default_rng(33)
    n = 768

    def mix(lo=-8, hi=-2, pzero=0.3):
        v = 10 ** rng.uniform(lo, hi, n)
        return np.where(rng.random(n) < pzero, 0.0, v)

    t = rng.uniform(215.0, 300.0, n)
    pres = rng.uniform(2e4, 1.02e5, n)
    rhodref = pres / (287.06 * t)
    exn = (pres / 1e5) ** (287.06 / 1004.71)
    tht = t / exn
    rv = 10 ** rng.uniform(-6, -1.8, n)
    rc, rr, ri, rs, rg = mix(), mix(), mix(), mix(), mix()
    cit = np.where(rng.random(n) < 0.4, 0.0, 10 ** rng.uniform(2, 6, n))
    ld = rng.random(n) < 0.9
    lsfact = rng.uniform(2400, 3200, n)
    lvfact = lsfact - rng.uniform(300, 400, n)
    cf = np.where(rng.random(n) < 0.3, 0.0, rng.uniform(0, 1, n))
    sigma_rc = rng.uniform(1e-7, 2e-4, n)
    hlc_hcf, hlc_hrc = rng.uniform(0, 1, n), mix(-7, -2, 0.3)
    hli_hcf, hli_hri = rng.uniform(0, 1, n), mix(-7, -2, 0.3)
    inp = dict(t=t, pres=pres, rhodref=rhodref, exn=exn, tht=tht, rv=rv, rc=rc, rr=rr, ri=ri, rs=rs, rg=rg,
               cit=cit, ld=ld.astype(np.float64), lsfact=lsfact, lvfact=lvfact, cf=cf, sigma_rc=sigma_rc,
               hlc_hcf=hlc_hcf, hlc_hrc=hlc_hrc, hli_hcf=hli_hcf, hli_hri=hli_hri)
    out = {}
    m = mods
    cit_new, rvheni, _ = m["nucl"].ice4_nucleation(tht, pres, rhodref, exn, lsfact, t, rv, cit, ld, True, ext)
    out.update(nucl_cit=cit_new, nucl_rvheni=rvheni)
    out["rrhong"] = m["rrhong"].ice4_rrhong(t, exn, lvfact, lsfact, tht, rr, ld, True, ext)
    out["rimltc"] = m["rimltc"].ice4_rimltc(t, exn, lvfact, lsfact, tht, ri, ld, True, ext)
    ssi, ka, dv, ai, cj = m["tend"].ice4_derived_fields(t, rhodref, pres, rv, ext)
    out.update(ssi=ssi, ka=ka, dv=dv, ai=ai, cj=cj)
    lbdar, lbdar_rf, lbdas, lbdag = m["tend"].ice4_slope_parameters(rhodref, t, rr, rs, rg, ext)
    out.update(lbdar=lbdar, lbdar_rf=lbdar_rf, lbdas=lbdas, lbdag=lbdag)
    # compute_pdf: reference enum 0=NONE 1=CLFR 2=ADJU 3=PDF (stencils/ice4_compute_pdf.py:42-44)
    for tag, rc_mode, ri_mode in (("pdf_sigm", 3, 0), ("none", 0, 0), ("clfr", 1, 1)):
        res = m["pdf"].ice4_compute_pdf(rhodref, rc, ri, cf, t, sigma_rc, ld, rc_mode, ri_mode, 0, ext)
        for nm, r in zip(("hlc_hcf", "hlc_lcf", "hlc_hrc", "hlc_lrc", "hli_hcf", "hli_lcf", "hli_hri", "hli_lri",
                          "rf"), res):
            out[f"pdf_{tag}_{nm}"] = r
    slow = m["slow"].ice4_slow(rhodref, t, ssi, rv, rc, ri, rs, rg, lbdas, lbdag, ai, cj, hli_hcf, hli_hri, ld,
                               False, ext)
    for nm, r in zip(("rchoni", "rvdeps", "riaggs", "riauts", "rvdepg"), slow):
        out[nm] = r
    warm = m["warm"].ice4_warm(rhodref, t, pres, tht, lbdar, lbdar_rf, ka, dv, cj, hlc_hcf, hlc_hrc, cf,
                               np.ones(n), rv, rc, rr, ld, False, 0, ext)
    for nm, r in zip(("rcautr", "rcaccr", "rrevav"), warm):
        out[nm] = r
    out["rcberi"] = m["ri"].ice4_fast_ri(rhodref, ai, cj, cit, ssi, rc, ri, ld, False, ext)
    fr, f1, f2 = m["rs"].compute_freezing_rate(rhodref, pres, dv, ka, cj, lbdas, t, rv, rs, slow[2], ld, False,
                                               True, ext)
    out.update(rs_freez=fr, rs_freez1=f1, rs_freez2=f2)
    # melting of snow with no riming/accretion inputs (rc = rr = 0 points only)
    z = np.zeros(n)
    out["rsmltg"], out["rcmltsr"] = m["rs"].conversion_melting_snow(rhodref, pres, dv, ka, cj, lbdas, t, rv, rs,
                                                                     z, z, ld & (rc == 0) & (rr == 0), False,
                                                                     True, ext)
    a, b, c = m["rg"].rain_contact_freezing(rhodref, lbdar, t, ri, rr, cit, ld, False, True, ext)
    out.update(ricfrrg=a, rrcfrig=b, ricfrr=c)
    rcdryg, ridryg, riwetg = m["rg"].cloud_pristine_collection_graupel(rhodref, lbdag, t, rc, ri, rg, ld, False,
                                                                      ext)
    out.update(rg_rcdryg=rcdryg, rg_ridryg=ridryg, rg_riwetg=riwetg)
    out["rgmltr"] = m["rg"].graupel_melting(rhodref, pres, dv, ka, cj, lbdag, t, rv, rg, rcdryg, z,
                                            ld & (rr == 0), False, True, ext)
    rec = {f"in_{k}": np.asarray(v, dtype=np.float64) for k, v in inp.items()}
    rec.update({f"out_{k}": np.asarray(v, dtype=np.float64) for k, v in out.items()})
    # rain fraction column sweep on a small grid (ng=1, nproma=16, nz=30)
    nk, nij = 30, 16
    prfr = rng.uniform(0, 1, (nk, nij)) * (rng.random((nk, nij)) < 0.5)
    prfr[-1, :] = 0.0
    r3 = [np.where(rng.random((nk, nij)) < 0.5, 0.0, 10 ** rng.uniform(-18, -12, (nk, nij))) for _ in range(3)]
    T = lambda a: _shim(np.ascontiguousarray(a.T[None]))
    res = m["ri_top"].ice4_rainfr_vert(T(prfr), T(r3[0]), T(r3[1]), T(r3[2]), ext)
    rec.update(rf_in_prfr=prfr, rf_in_rr=r3[0], rf_in_rs=r3[1], rf_in_rg=r3[2],
               rf_out_prfr=np.asarray(res)[0].T.copy())
    return {"processes": rec}


def warm_subg_case(mods, Phyex):
    """ICE4_WARM with the subgrid evaporation options CLFR (1) and PRFR (2)
    (src/ice3/jax/stencils/ice4_warm.py:15), hard pass, on seeded random
    points; lbdar_rf is formed from the precipitation fraction as
    mode_ice4_tendencies.F90 forms it (LBR (rho max(rr / rf, R_RTMIN))^LBEXR)."""
    ext = dict(Phyex("AROME", TSTEP=DT).to_externals())
    rng = np.random.default_rng(44)
    n = 1024

    def mix(lo=-8, hi=-2, pzero=0.3):
        v = 10 ** rng.uniform(lo, hi, n)
        return np.where(rng.random(n) < pzero, 0.0, v)

    t = rng.uniform(250.0, 305.0, n)
    pres = rng.uniform(3e4, 1.02e5, n)
    rhodref = pres / (287.06 * t)
    exn = (pres / 1e5) ** (287.06 / 1004.71)
    tht = t / exn
    rv = 10 ** rng.uniform(-5, -1.8, n)
    rc, rr = mix(), mix(pzero=0.2)
    ld = rng.random(n) < 0.9
    cf = np.where(rng.random(n) < 0.3, 0.0, rng.uniform(0, 1, n))
    rf = np.where(rng.random(n) < 0.2, 0.0, rng.uniform(0, 1, n))
    hlc_hcf, hlc_hrc = rng.uniform(0, 1, n), mix(-7, -2, 0.3)
    ssi, ka, dv, ai, cj = mods["tend"].ice4_derived_fields(t, rhodref, pres, rv, ext)
    lbdar, _, _, _ = mods["tend"].ice4_slope_parameters(rhodref, t, rr, np.zeros(n), np.zeros(n), ext)
    lbdar = np.asarray(lbdar, dtype=np.float64)
    lbdar_rf = np.where((rr > 0) & (rf > 0),
                        ext["LBR"] * (rhodref * np.maximum(rr / np.where(rf > 0, rf, 1.0), ext["R_RTMIN"]))
                        ** ext["LBEXR"], 0.0)
    rec = dict(in_t=t, in_pres=pres, in_rhodref=rhodref, in_tht=tht, in_rv=rv, in_rc=rc, in_rr=rr,
               in_ld=ld.astype(np.float64), in_cf=cf, in_rf=rf, in_hlc_hcf=hlc_hcf, in_hlc_hrc=hlc_hrc,
               in_ssi=ssi, in_ka=ka, in_dv=dv, in_ai=ai, in_cj=cj, in_lbdar=lbdar, in_lbdar_rf=lbdar_rf)
    for mode in (1, 2):
        res = mods["warm"].ice4_warm(rhodref, t, pres, tht, lbdar, lbdar_rf, ka, dv, cj, hlc_hcf, hlc_hrc, cf, rf,
                                     rv, rc, rr, ld, False, mode, ext)
        for nm, r in zip(("rcautr", "rcaccr", "rrevav"), res):
            rec[f"out{mode}_{nm}"] = r
    return {"warm_subg": rec}


def rain_ice_pieces_case(Phyex):
    """The RAIN_ICE / ICE4_STEPPING stencils of the reference JAX on seeded
    random points (src/ice3/jax/stencils/rain_ice.py:19, :95, :141, :323;
    stencils/ice4_tendencies.py:330; stencils/ice4_stepping.py:59, :109,
    :232; stencils/ice4_correct_negativities.py:14).

    Where the JAX stencil and the Fortran ICE4_STEPPING differ (the JAX
    depletion limit is the time to reach XRTMIN from (r_min - r - b) / a for
    growing or present species; the Fortran one the time to reach zero of a
    present, depleting species), the inputs are drawn inside the set where
    both give the same answer: every r > 0, instantaneous changes b >= 0,
    vapour never depleting, thresholds r_min = 0 passed to the JAX.  The JAX
    negativity correction refills vapour from snow and graupel only, up to
    their own minima: case A has vapour far above every threshold (the
    Fortran refill lines do nothing), case B pins the JAX form itself."""
    import ice3.jax.stencils.ice4_correct_negativities as neg
    import ice3.jax.stencils.ice4_stepping as stp
    import ice3.jax.stencils.ice4_tendencies as tend
    import ice3.jax.stencils.rain_ice as rit

    ext = dict(Phyex("AROME", TSTEP=DT).to_externals())
    rng = np.random.default_rng(55)
    n = 1024
    rec = {}

    def mix(lo=-8, hi=-2, pzero=0.3, size=n):
        v = 10 ** rng.uniform(lo, hi, size)
        return np.where(rng.random(size) < pzero, 0.0, v)

    # thermo + mask
    t = rng.uniform(215.0, 305.0, n)
    exn = rng.uniform(0.6, 1.02, n)
    th = t / exn
    r = {k: mix() for k in ("rv", "rc", "rr", "ri", "rs", "rg")}
    r["rv"] = 10 ** rng.uniform(-6, -1.8, n)
    for k in ("rc", "rr", "ri", "rs", "rg"):        # a few values right at and below the thresholds
        r[k] = np.where(rng.random(n) < 0.05, ext[k[1].upper() + "_RTMIN"] * rng.choice([0.5, 1.0, 2.0], n), r[k])
    ls, lv = rit.rain_ice_thermo(_shim(exn), _shim(th), *(_shim(r[k]) for k in ("rv", "rc", "rr", "ri", "rs", "rg")),
                                 ext)
    mask = rit.rain_ice_mask(*(_shim(r[k]) for k in ("rc", "rr", "ri", "rs", "rg")), ext)
    rec.update(th_exn=exn, th_th=th, **{f"th_{k}": v for k, v in r.items()}, th_out_ls=ls, th_out_lv=lv,
               th_out_mask=np.asarray(mask, dtype=np.float64))

    # total tendencies: end-of-step values near the start values
    names = ("th", "v", "c", "r", "i", "s", "g")
    r0 = {"th": th, "v": r["rv"], "c": r["rc"], "r": r["rr"], "i": r["ri"], "s": r["rs"], "g": r["rg"]}
    wr = {k: v * (1.0 + rng.uniform(-0.5, 0.5, n)) for k, v in r0.items()}
    src = {k: rng.uniform(-1e-6, 1e-6, n) for k in names}
    src["th"] = rng.uniform(-1e-2, 1e-2, n)
    rvheni = mix(-12, -7, 0.5)
    lsx, lvx = np.asarray(ls) / exn, np.asarray(lv) / exn
    ext_t = dict(ext, INV_TSTEP=1.0 / DT)
    res = rit.rain_ice_total_tendencies(*(_shim(wr[k]) for k in names), _shim(lsx), _shim(lvx), _shim(exn),
                                        *(_shim(src[k]) for k in names), _shim(rvheni),
                                        *(_shim(r0[k]) for k in names[1:]), ext_t)
    rec.update({f"tt_wr_{k}": wr[k] for k in names})
    rec.update({f"tt_src_{k}": src[k] for k in names})
    rec.update(tt_rvheni=rvheni, tt_lsx=lsx, tt_lvx=lvx)
    for k, v in zip(("th", "v", "c", "r", "i", "s", "g"), res[7:]):
        rec[f"tt_out_{k}"] = np.asarray(v, dtype=np.float64)

    # fog deposition on the lowest level of (1, n, 2) columns
    rcs3 = rng.uniform(-1e-7, 1e-6, (1, n, 2))
    rct3 = np.stack([mix(-8, -3, 0.3), mix(-8, -3, 0.3)], axis=-1)[None]
    rho3 = rng.uniform(0.3, 1.3, (1, n, 2))
    dz3 = rng.uniform(10.0, 300.0, (1, n, 2))
    inprc = rng.uniform(0.0, 1e-6, (1, n))
    fr, fi = rit.fog_deposition(_shim(rcs3), _shim(rct3), _shim(rho3), _shim(dz3), _shim(inprc), ext)
    rec.update(fog_rcs=rcs3[0, :, 0], fog_rct=rct3[0, :, 0], fog_rho=rho3[0, :, 0], fog_dzz=dz3[0, :, 0],
               fog_inprc=inprc[0], fog_out_rcs=np.asarray(fr)[0, :, 0], fog_out_inprc=np.asarray(fi)[0])

    # aggregation of one pass
    rate_names = ("rchoni", "rvdeps", "riaggs", "riauts", "rvdepg", "rcautr", "rcaccr", "rrevav", "rcberi",
                  "rsmltg", "rcmltsr", "rraccss", "rraccsg", "rsaccrg", "rcrimss", "rcrimsg", "rsrimcg",
                  "ricfrrg", "rrcfrig", "ricfrr", "rcwetg", "riwetg", "rrwetg", "rswetg", "rcdryg", "ridryg",
                  "rrdryg", "rsdryg", "rgmltr")
    rates = {k: mix(-12, -5, 0.4) for k in rate_names}
    rates["rvdeps"] = np.where(rng.random(n) < 0.3, -rates["rvdeps"], rates["rvdeps"])   # sublimation
    rates["rvdepg"] = np.where(rng.random(n) < 0.3, -rates["rvdepg"], rates["rvdepg"])
    z = np.zeros(n)
    res = tend.ice4_total_tendencies_update(_shim(lsx), _shim(lvx), *([_shim(z)] * 7),
                                            *(_shim(rates[k]) for k in rate_names))
    rec.update({f"ag_{k}": v for k, v in rates.items()})
    rec.update(ag_ls=lsx, ag_lv=lvx)
    for k, v in zip(names, res):
        rec[f"ag_out_{k}"] = np.asarray(v, dtype=np.float64)

    # step limiter and state update
    sp = ("c", "r", "i", "s", "g")
    rt = {k: 10 ** rng.uniform(-9, -3, n) for k in sp}
    a = {k: np.where(rng.random(n) < 0.2, 0.0, rng.choice([-1.0, 1.0], n) * 10 ** rng.uniform(-9, -5, n))
         for k in sp}
    b = {k: np.where(rng.random(n) < 0.5, 0.0, 10 ** rng.uniform(-10, -4, n)) for k in sp}
    a_th = np.where(rng.random(n) < 0.2, 0.0, rng.uniform(-2e-3, 2e-3, n))
    b_th = np.where(rng.random(n) < 0.5, 0.0, rng.uniform(-0.5, 0.5, n))
    th_s = ext["TT"] / exn + rng.uniform(-1.0, 1.0, n)          # around the 0 C crossing
    t_micro = np.where(rng.random(n) < 0.5, 0.0, rng.uniform(0.0, DT, n))
    ld = rng.random(n) < 0.9
    ext0 = dict(ext, C_RTMIN=0.0, R_RTMIN=0.0, I_RTMIN=0.0, S_RTMIN=0.0, G_RTMIN=0.0)
    dtm, ld_new = stp.ice4_step_limiter(_shim(exn), _shim(th_s), _shim(a_th), _shim(b_th),
                                        *(_shim(rt[k]) for k in sp), *(_shim(a[k]) for k in sp),
                                        *(_shim(b[k]) for k in sp), _shim(t_micro), ld, DT, ext0)
    rec.update(sl_exn=exn, sl_th=th_s, sl_a_th=a_th, sl_b_th=b_th, sl_t_micro=t_micro,
               sl_ld=ld.astype(np.float64), sl_out_dt=np.asarray(dtm, dtype=np.float64),
               sl_out_ld=np.asarray(ld_new, dtype=np.float64))
    rec.update({f"sl_r{k}": rt[k] for k in sp})
    rec.update({f"sl_a{k}": a[k] for k in sp})
    rec.update({f"sl_b{k}": b[k] for k in sp})
    ci = np.where(rng.random(n) < 0.3, 0.0, 10 ** rng.uniform(2, 6, n))
    rt_u = {k: np.where(rng.random(n) < 0.2, -rt[k] * 0.5, rt[k]) for k in sp}    # some depletions below zero
    res = stp.state_update(_shim(th_s), _shim(a_th), _shim(b_th), *(_shim(rt_u[k]) for k in sp),
                           *(_shim(a[k]) for k in sp), *(_shim(-np.abs(b[k])) for k in sp), _shim(ci),
                           _shim(np.asarray(dtm)), ld)
    rec.update({f"su_r{k}": rt_u[k] for k in sp})
    rec.update(su_ci=ci)
    for k, v in zip(("th", "c", "r", "i", "s", "g", "ci"), res):
        rec[f"su_out_{k}"] = np.asarray(v, dtype=np.float64)

    # negativity correction, case A (vapour far above every threshold) and B (vapour near zero)
    for case, rv_neg in (("A", 10 ** rng.uniform(-5, -2, n)), ("B", rng.uniform(-1e-9, 1e-14, n))):
        # case A: the negative parts (at most 5e-6 in all) stay below the vapour (at least 1e-5)
        hi = -6.0 if case == "A" else -4.0
        x = {k: rng.choice([-1.0, 1.0], n) * mix(-10, hi, 0.2) for k in ("rc", "rr", "ri", "rs", "rg")}
        if case == "B":
            for k in ("rs", "rg"):
                x[k] = np.abs(x[k])
        th_n = rng.uniform(250.0, 320.0, n)
        res = neg.ice4_correct_negativities(_shim(th_n), _shim(rv_neg), *(_shim(x[k]) for k in ("rc", "rr", "ri",
                                            "rs", "rg")), _shim(lvx), _shim(lsx), ext)
        rec.update({f"cn{case}_{k}": v for k, v in x.items()})
        rec.update({f"cn{case}_th": th_n, f"cn{case}_rv": rv_neg})
        for k, v in zip(("th", "rv", "rc", "rr", "ri", "rs", "rg"), res):
            rec[f"cn{case}_out_{k}"] = np.asarray(v, dtype=np.float64)
    rec["cn_lsx"], rec["cn_lvx"] = lsx, lvx
    return {"ri_pieces": rec}


def reference_fixture_states():
    """The ice_adjust states of the reference's own component tests
    (tests/components/test_ice_adjust_jax.py): `simple_test_data` (:30-69),
    `realistic_test_data` (:72-151) and the supersaturated state of
    `test_cloud_formation` (:285-318), restated with numpy; timestep 60 s,
    Phyex("AROME", TSTEP=60)."""
    zero = ("rc", "ri", "rr", "rs", "rg", "cf_mf", "rc_mf", "ri_mf", "rvs", "rcs", "ris", "ths")

    def uniform(shape, th, rv):
        st = dict(sigqsat=np.full(shape, 0.01), pabs=np.full(shape, 85000.0), sigs=np.full(shape, 0.1),
                  th=np.full(shape, th), exn=np.full(shape, 0.95), exn_ref=np.full(shape, 0.95),
                  rho_dry_ref=np.ones(shape), rv=np.full(shape, rv))
        st.update({k: np.zeros(shape) for k in zero})
        return st

    nx, ny, nz = 10, 10, 20
    z = np.linspace(0.0, 10000.0, nz)
    p0, t0, gamma = 101325.0, 288.15, 0.0065
    pabs = np.tile(p0 * (1 - gamma * z / t0) ** 5.26, (nx, ny, 1))
    temp = np.tile(t0 - gamma * z, (nx, ny, 1))
    exn = (pabs / 100000.0) ** (287.0 / 1004.0)
    real = dict(sigqsat=np.full((nx, ny, nz), 0.01), pabs=pabs, sigs=np.full((nx, ny, nz), 0.1), th=temp / exn,
                exn=exn, exn_ref=exn, rho_dry_ref=pabs / (287.0 * temp),
                rv=np.tile(0.015 * np.exp(-z / 2000.0), (nx, ny, 1)),
                rc=np.where(np.tile((z > 2000.0) & (z < 6000.0), (nx, ny, 1)), 0.001, 0.0),
                ri=np.where(np.tile(z > 5000.0, (nx, ny, 1)), 0.0005, 0.0))
    real.update({k: np.zeros((nx, ny, nz)) for k in zero if k not in ("rc", "ri")})
    return {"simple": uniform((5, 5, 10), 285.0, 0.010), "realistic": real,
            "cloud_formation": uniform((5, 5, 10), 280.0, 0.020)}


def ia_fixtures_case(IceAdjustJAX, Phyex):
    """IceAdjustJAX (jit off) on the reference test states, timestep 60 s."""
    ia = IceAdjustJAX(Phyex("AROME", TSTEP=60.0), jit=False)
    names = ("t", "rv_out", "rc_out", "ri_out", "cldfr", "hlc_hrc", "hlc_hcf", "hli_hri", "hli_hcf", "cph", "lv",
             "ls", "rvs", "rcs", "ris", "ths")
    rec = {}
    for cname, st in reference_fixture_states().items():
        res = ia(**{k: _shim(v) for k, v in st.items()}, timestep=60.0)
        for k, v in st.items():
            rec[f"{cname}_in_{k}"] = v
        for n, r in zip(names, res):
            rec[f"{cname}_out_{n}"] = np.asarray(r, dtype=np.float64)
    return {"ia_fixtures": rec}


def adjoint_fd_case(IceAdjustJAX, sedimentation_stat, Phyex):
    """Reference directional derivatives for the adjoint checks: centred
    differences (h = 1e-7, relative directions N(0,1)|x|) of the reference's
    own IceAdjustJAX and sedimentation_stat run in FP64.  ice_adjust: 32
    columns x 90 levels, N(0,1) cotangents on T, rv, rc, ri and cloud
    fraction (sigqsat held fixed), the sources scaled by U[0.5, 1.5] off the
    kink of the source limiter; J = <g, y> per point at x + h dx, x, x - h dx.
    Sedimentation (JAX semantics): 24 columns, cotangents on the five sources
    and the surface precipitation, J per column."""
    from ice3gb.state import make_state
    h = 1e-7
    rec = {}
    ia = IceAdjustJAX(Phyex("AROME", TSTEP=DT), jit=False)
    st = _np(make_state(32, 90, seed=31, precip=True))
    rng = np.random.default_rng(66)
    ins = ("sigqsat", "pabs", "sigs", "th", "exn", "exn_ref", "rho_dry_ref", "rv", "rc", "ri", "rr", "rs", "rg",
           "cf_mf", "rc_mf", "ri_mf", "rvs", "rcs", "ris", "ths")
    outs = ("t", "rv_out", "rc_out", "ri_out", "cldfr", "hlc_hrc", "hlc_hcf", "hli_hri", "hli_hcf", "cph", "lv",
            "ls", "rvs", "rcs", "ris", "ths")
    shape = st["th"].shape
    x = {k: st[k] for k in ins if k != "sigqsat"}
    x["sigqsat"] = np.broadcast_to(st["sigqsat"][None, :], shape).copy()
    for k in ("rvs", "rcs", "ris", "ths"):
        x[k] = x[k] * rng.uniform(0.5, 1.5, shape)
    dx = {k: rng.standard_normal(shape) * np.abs(v) for k, v in x.items()}
    dx["sigqsat"][:] = 0.0
    g = {k: rng.standard_normal(shape) for k in ("t", "rv_out", "rc_out", "ri_out", "cldfr")}

    def j_ia(xx):
        y = dict(zip(outs, ia(**{k: _shim(v) for k, v in xx.items()}, timestep=DT)))
        return sum(g[k] * np.asarray(y[k], dtype=np.float64) for k in g)
    for tag, sgn in (("p", 1.0), ("0", 0.0), ("m", -1.0)):
        rec[f"ia_j{tag}"] = j_ia({k: v + sgn * h * dx[k] for k, v in x.items()})
    rec.update({f"ia_x_{k}": v for k, v in x.items()})
    rec.update({f"ia_dx_{k}": v for k, v in dx.items()})
    rec.update({f"ia_g_{k}": v for k, v in g.items()})

    ext = dict(Phyex("AROME", TSTEP=DT).to_externals())
    ext.update(LBC_LAND=ext["LBC_1"], LBC_SEA=ext["LBC_2"], FSEDC_LAND=ext["FSEDC_1"], FSEDC_SEA=ext["FSEDC_2"])
    st = _np(make_state(24, 90, seed=32, precip=True))
    nk, nij = st["pabs"].shape
    sx = {"rhodref": st["rho_dry_ref"], "dzz": st["dzz"], "pabs": st["pabs"], "tht": st["th"]}
    for k, r in (("rcs", "rc"), ("rrs", "rr"), ("ris", "ri"), ("rss", "rs"), ("rgs", "rg")):
        sx[k] = st[r] / DT * rng.uniform(0.5, 1.5, (nk, nij))
    sdx = {k: rng.standard_normal((nk, nij)) * np.abs(v) for k, v in sx.items()}
    src = ("rcs", "rrs", "ris", "rss", "rgs")
    gs = {k: rng.standard_normal((nk, nij)) for k in src}
    gp = {k: rng.standard_normal(nij) for k in ("inprc", "inprr", "inpri", "inprs", "inprg")}
    z = np.zeros(nij)
    T = lambda a: _shim(np.ascontiguousarray(a.T[None, :, :]))

    def j_sed(xx):
        res = sedimentation_stat(*(T(xx[k]) for k in ("rhodref", "dzz", "pabs", "tht") + src), _shim(z[None, :, None]),
                                 _shim(z[None, :, None]), ext)
        y = [np.asarray(r, dtype=np.float64)[0] for r in res]
        j = sum((gs[k] * y[i].T).sum(axis=0) for i, k in enumerate(src))
        return j + sum(gp[k] * y[10 + i] for i, k in enumerate(gp))
    for tag, sgn in (("p", 1.0), ("0", 0.0), ("m", -1.0)):
        rec[f"sed_j{tag}"] = j_sed({k: v + sgn * h * sdx[k] for k, v in sx.items()})
    rec.update({f"sed_x_{k}": v for k, v in sx.items()})
    rec.update({f"sed_dx_{k}": v for k, v in sdx.items()})
    rec.update({f"sed_g_{k}": v for k, v in {**gs, **gp}.items()})
    return {"adjoint_fd": rec}


def src_1d_case():
    """The SRC_1D table of the reference (src/ice3/phyex_common/lookup_table.py:4)."""
    from ice3.phyex_common.lookup_table import SRC_1D
    return {"src_1d": {"SRC_1D": np.asarray(SRC_1D, dtype=np.float64)}}


def tiwmx_case(Phyex):
    """The reference's saturation pressures (src/ice3/jax/functions/tiwmx.py:18,60)
    on the grid of PHYEX's TIWMX tables, T = j/100 K (micro/modd_tiwmx.F90):
    a stride through 13200..37316 and every entry around 273.15 K, where
    ESTABI switches from the ice to the water formula."""
    from ice3.jax.functions.tiwmx import e_sat_i, e_sat_w
    ext = Phyex("AROME").to_externals()
    j = np.unique(np.concatenate([np.arange(13200, 37317, 37), np.arange(27300, 27330), [37316]]))
    t = _shim(j / 100.0)
    return {"tiwmx": {"j": j.astype(np.float64), "esw": np.asarray(e_sat_w(t, ext), dtype=np.float64),
                      "esi": np.asarray(e_sat_i(t, ext), dtype=np.float64)}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference-src", default=os.environ.get("ICE3GB_REFERENCE_SRC"),
                    required="ICE3GB_REFERENCE_SRC" not in os.environ,
                    help="the reference's src/ directory (or set ICE3GB_REFERENCE_SRC)")
    ap.add_argument("--only", nargs="*", default=None, help="write only these golden files (names without .npz)")
    args = ap.parse_args()
    import refshim

    refshim.install()
    sys.path.insert(0, args.reference_src)
    np.seterr(all="ignore")
    from ice3.jax.ice_adjust import IceAdjustJAX
    from ice3.jax.stencils.sedimentation import sedimentation_stat
    from ice3.phyex_common.phyex import Phyex
    import ice3.jax.stencils.ice4_nucleation as nucl
    import ice3.jax.stencils.ice4_rrhong as rrhong
    import ice3.jax.stencils.ice4_rimltc as rimltc
    import ice3.jax.stencils.ice4_tendencies as tend
    import ice3.jax.stencils.ice4_compute_pdf as pdf
    import ice3.jax.stencils.ice4_slow as slow
    import ice3.jax.stencils.ice4_warm as warm
    import ice3.jax.stencils.ice4_fast_ri as fri
    import ice3.jax.stencils.ice4_fast_rs as frs
    import ice3.jax.stencils.ice4_fast_rg as frg
    import ice3.jax.stencils.rain_ice as ri_top

    mods = dict(nucl=nucl, rrhong=rrhong, rimltc=rimltc, tend=tend, pdf=pdf, slow=slow, warm=warm, ri=fri,
                rs=frs, rg=frg, ri_top=ri_top)
    blobs = {}
    blobs.update(ice_adjust_cases(IceAdjustJAX, Phyex))
    blobs.update(sedimentation_case(sedimentation_stat, Phyex))
    blobs.update(process_cases(mods, Phyex))
    blobs.update(warm_subg_case(mods, Phyex))
    blobs.update(src_1d_case())
    blobs.update(tiwmx_case(Phyex))
    blobs.update(rain_ice_pieces_case(Phyex))
    blobs.update(ia_fixtures_case(IceAdjustJAX, Phyex))
    blobs.update(adjoint_fd_case(IceAdjustJAX, sedimentation_stat, Phyex))
    for name, rec in blobs.items():
        if args.only is not None and name not in args.only:
            continue
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **{k: np.asarray(v, dtype=np.float64) for k, v in rec.items()})
        print(f"wrote {path} ({os.path.getsize(path) / 1e3:.0f} kB)")


if __name__ == "__main__":
    main()
