"""ctypes wrapper of the CPU oracle (oracle/ice3_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by the CPU-baseline leg of bench.py, always as the checker.  The product
never imports this module.

Arrays are numpy float64, [nk, nij] C-contiguous (= the ABI's [nk][nij]).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys
import time
from typing import Dict, Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_REPO = os.path.dirname(_HERE)
_PKG = os.path.join(_REPO, "dwarf-p-ice3_gb300")
if _PKG not in sys.path:
    sys.path.insert(0, _PKG)

from ice3gb._abi import (IceAdjustFields, RainIceFields, RainIceOptions, SedimentationFields, StepFields,  # noqa: E402
                         STEP_IN, STEP_INOUT, STEP_OUT2, STEP_OUT3)
from ice3gb.constants import ConstantsTable, Ice3gbConstants, Ice3gbLuts  # noqa: E402

LIB_PATH = os.path.join(_HERE, "_build", "libice3_oracle.so")
_lib = None

IA_IN = ("sigqsat", "pabs", "sigs", "th", "exn", "exn_ref", "rho_dry_ref", "rv", "rc", "ri", "rr", "rs", "rg",
         "cf_mf", "rc_mf", "ri_mf")
IA_INOUT = ("rvs", "rcs", "ris", "ths")
IA_OUT = ("t", "rv_out", "rc_out", "ri_out", "cldfr", "hlc_hrc", "hlc_hcf", "hli_hri", "hli_hcf", "cph", "lv", "ls")
# order of the reference's 16-tuple (src/ice3/jax/stencils/ice_adjust.py:381-398)
IA_RESULT = IA_OUT + IA_INOUT

NBU_NAMES = ("rvheni_mr", "rrhong_mr", "rimltc_mr", "rsrimcg_mr", "rchoni", "rvdeps", "riaggs", "riauts",
             "rvdepg", "rcautr", "rcaccr", "rrevav", "rcrimss", "rcrimsg", "rsrimcg", "rraccss", "rraccsg",
             "rsaccrg", "rsmltg", "rcmltsr", "ricfrrg", "rrcfrig", "ricfrr", "rcwetg", "riwetg", "rrwetg",
             "rswetg", "rcdryg", "ridryg", "rrdryg", "rsdryg", "rgmltr", "rcberi",
             # hail (KRR = 7)
             "rwetgh", "rwetgh_mr", "rcweth", "riweth", "rsweth", "rgweth", "rrweth", "rcdryh", "ridryh",
             "rsdryh", "rrdryh", "rgdryh", "rdryhg", "rhmltr",
             # OCND2 (ICE4_FAST_RI_RS)
             "rvdepi", "rilars")
RS_NAMES = ("rcrims", "rcrimss", "rsrimcg", "rraccs", "rraccss", "rsaccrg", "freez1", "freez2")
RG_NAMES = ("rcdryg", "ridryg", "riwetg", "rsdryg", "rswetg", "rrdryg", "freez1", "freez2")


def build(force: bool = False) -> str:
    src = os.path.join(_HERE, "ice3_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return LIB_PATH


def load():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.ice3o_budget_count.restype = ctypes.c_int
        assert _lib.ice3o_budget_count() == len(NBU_NAMES)
    return _lib


def _ptr(a: Optional[np.ndarray]):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.c_void_p)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def ice_adjust(table: ConstantsTable, st: Dict[str, np.ndarray], dt: float, srcs: bool = False
               ) -> Dict[str, np.ndarray]:
    """Oracle ice_adjust; returns the 16 outputs keyed by name (and "srcs",
    PSRCS, when asked)."""
    lib = load()
    ins = {k: _f64(st[k]) for k in IA_IN}
    nk, nij = ins["pabs"].shape
    io = {k: _f64(st[k]).copy() for k in IA_INOUT}
    out = {k: np.empty((nk, nij)) for k in IA_OUT}
    if srcs:
        out["srcs"] = np.empty((nk, nij))
    f = IceAdjustFields()
    for k, v in {**ins, **io, **out}.items():
        setattr(f, k, _ptr(v))
    f.sigqsat_3d = 1 if ins["sigqsat"].ndim == 2 else 0
    if table.values["OCND2"] != 0.0:
        # separate liquid and ice clouds: heights, the per-column ice cloud
        # weight, and five more outputs (condensation.F90:373-395, :588-637)
        ins["zz"] = _f64(st["zz"])
        ins["ice_cld_wgt"] = _f64(st["ice_cld_wgt"])
        f.zz, f.ice_cld_wgt = _ptr(ins["zz"]), _ptr(ins["ice_cld_wgt"])
        for k in ("icldfr", "wcldfr", "ssio", "ssiu", "ifr"):
            out[k] = np.empty((nk, nij))
            setattr(f, k, _ptr(out[k]))
    rc = lib.ice3o_ice_adjust(ctypes.byref(table.consts), nij, nk, ctypes.c_double(dt), ctypes.byref(f))
    if rc != 0:
        raise RuntimeError(f"oracle ice_adjust returned {rc}")
    return {**out, **io}


def tiwmx_tables(table: ConstantsTable):
    """The oracle's TIWMX saturation tables (ESTABW, ESTABI) at T = j/100 K,
    j = 13200..37316 (micro/mode_ini_tiwmx.F90)."""
    lib = load()
    n = lib.ice3o_tiwmx_size()
    w, i = np.empty(n), np.empty(n)
    lib.ice3o_tiwmx_tables(ctypes.byref(table.consts), _ptr(w), _ptr(i))
    return w, i


def src_1d() -> np.ndarray:
    """The oracle's SRC_1D table (condensation.F90 index -22..11)."""
    lib = load()
    lib.ice3o_src_1d.restype = ctypes.c_double
    lib.ice3o_src_1d.argtypes = [ctypes.c_int]
    return np.array([lib.ice3o_src_1d(i) for i in range(-22, 12)])


def sedimentation(table: ConstantsTable, st: Dict[str, np.ndarray], dt: float, fortran: bool,
                  with_fpr: bool = False) -> Dict[str, np.ndarray]:
    lib = load()
    rho = _f64(st["rhodref"])
    nk, nij = rho.shape
    f = SedimentationFields()
    keep = {}
    for k in ("rhodref", "dzz", "pabs", "tht"):
        keep[k] = _f64(st[k])
        setattr(f, k, _ptr(keep[k]))
    for k in ("sea", "town"):
        if st.get(k) is not None:
            keep[k] = _f64(st[k])
            setattr(f, k, _ptr(keep[k]))
    out = {}
    for k in ("rcs", "rrs", "ris", "rss", "rgs"):
        out[k] = _f64(st[k]).copy()
        setattr(f, k, _ptr(out[k]))
    for k in ("inprc", "inprr", "inpri", "inprs", "inprg"):
        out[k] = np.empty(nij)
        setattr(f, k, _ptr(out[k]))
    if with_fpr:
        for k in ("fpr_c", "fpr_r", "fpr_i", "fpr_s", "fpr_g"):
            out[k] = np.empty((nk, nij))
            setattr(f, k, _ptr(out[k]))
    f.fortran_semantics = 1 if fortran else 0
    rc = lib.ice3o_sedimentation(ctypes.byref(table.consts), nij, nk, ctypes.c_double(dt), ctypes.byref(f))
    if rc != 0:
        raise RuntimeError(f"oracle sedimentation returned {rc}")
    return out


RI_IN = ("exn", "dzz", "rhodref", "exnref", "pabs", "cldfr", "sigs", "tht", "rvt", "rct", "rrt", "rit", "rst",
         "rgt")
RI_INOUT = ("cit", "hlc_hrc", "hlc_hcf", "hli_hri", "hli_hcf", "ths", "rvs", "rcs", "rrs", "ris", "rss", "rgs")
RI_OUT3 = ("evap3d", "rainfr")
RI_OUT2 = ("inprc", "inprr", "inpri", "inprs", "inprg", "indep")


def rain_ice(table: ConstantsTable, st: Dict[str, np.ndarray], dt: float, lsedim_after: int = -1,
             ldeposc: int = -1, lfeedbackt: int = -1, max_passes: int = 0, sed_jax: int = 0,
             with_fpr: bool = False, with_ties: bool = False):
    """Oracle rain_ice on ABI-named fields; returns (outputs dict, status bits).
    with_ties: also out["tie"], the bits of the sub-stepping's decisions on
    rounding residuals (ice3o_rain_ice_ties): 1 a graupel or hail growth
    mode, 2 the CIT reset after an ice residual, 4 an MRSTEP threshold on
    the chosen sub-step, 8 a hard pass after such a CIT reset."""
    lib = load()
    keep = {k: _f64(st[k]) for k in RI_IN}
    nk, nij = keep["exn"].shape
    f = RainIceFields()
    for k, v in keep.items():
        setattr(f, k, _ptr(v))
    for k in ("sea", "town"):
        if st.get(k) is not None:
            keep[k] = _f64(st[k])
            setattr(f, k, _ptr(keep[k]))
    out = {k: _f64(st[k]).copy() for k in RI_INOUT}
    out.update({k: np.empty((nk, nij)) for k in RI_OUT3})
    out.update({k: np.empty(nij) for k in RI_OUT2})
    if table.values["OCND2"] != 0.0:
        # OCND2: the ice_adjust OCND2 outputs of the same state
        for k in ("ssio", "ssiu", "ifr", "icldfr"):
            keep[k] = _f64(st[k])
            setattr(f, k, _ptr(keep[k]))
    hail = table.values["NRR"] == 7.0
    if hail:
        # hail (KRR = 7): mixing ratio at t, in-out source, precipitation
        keep["rht"] = _f64(st["rht"])
        f.rht = _ptr(keep["rht"])
        out["rhs"] = _f64(st["rhs"]).copy()
        out["inprh"] = np.empty(nij)
    if with_fpr:
        out.update({k: np.empty((nk, nij)) for k in ("fpr_c", "fpr_r", "fpr_i", "fpr_s", "fpr_g")})
        if hail:
            out["fpr_h"] = np.empty((nk, nij))
    for k, v in out.items():
        setattr(f, k, _ptr(v))
    opt = RainIceOptions(lsedim_after, ldeposc, lfeedbackt, max_passes, sed_jax)
    bits = ctypes.c_uint32(0)
    lib.ice3o_rain_ice.argtypes = [ctypes.POINTER(Ice3gbConstants), ctypes.POINTER(Ice3gbLuts), ctypes.c_int,
                                   ctypes.c_int, ctypes.c_double, ctypes.POINTER(RainIceOptions),
                                   ctypes.POINTER(RainIceFields), ctypes.POINTER(ctypes.c_uint32)]
    tie = np.zeros((nk, nij), dtype=np.uint8) if with_ties else None
    lib.ice3o_rain_ice_ties.argtypes = lib.ice3o_rain_ice.argtypes + [ctypes.c_void_p]
    rc = lib.ice3o_rain_ice_ties(ctypes.byref(table.consts), ctypes.byref(table.luts), nij, nk, dt,
                                 ctypes.byref(opt), ctypes.byref(f), ctypes.byref(bits),
                                 None if tie is None else tie.ctypes.data_as(ctypes.c_void_p))
    if rc != 0:
        raise RuntimeError(f"oracle rain_ice returned {rc}")
    if with_ties:
        out["tie"] = tie
    return out, bits.value


def rain_ice_depletion_alternatives(table: ConstantsTable, st: Dict[str, np.ndarray], dt: float,
                                    masks=(1, 2, 3), **kw):
    """Oracle rain_ice with other outcomes of its depletion ties: for each bit
    mask, the k-th rounding-decided MNH_TINY-pass decision of every point
    (bit k-1 set) takes the other branch (ice3o_set_depletion_flip).  Returns
    the list of output dicts, one per mask."""
    lib = load()
    outs = []
    try:
        for m in masks:
            lib.ice3o_set_depletion_flip(int(m))
            outs.append(rain_ice(table, st, dt, **kw)[0])
    finally:
        lib.ice3o_set_depletion_flip(0)
    return outs


def physics_step_depletion_alternatives(table: ConstantsTable, st: Dict[str, np.ndarray], dt: float,
                                        masks=(1, 2, 3), **kw):
    """physics_step with the depletion-tie outcomes of
    rain_ice_depletion_alternatives."""
    lib = load()
    outs = []
    try:
        for m in masks:
            lib.ice3o_set_depletion_flip(int(m))
            outs.append(physics_step(table, st, dt, **kw)[0])
    finally:
        lib.ice3o_set_depletion_flip(0)
    return outs


# ---- per-process entry points (hard pass) --------------------------------

def nucleation(table, tht, pabst, rhodref, exn, lsfact, t, rvt, cit, ldcompute):
    lib = load()
    a = [_f64(x).ravel() for x in (tht, pabst, rhodref, exn, lsfact, t, rvt)]
    cit = _f64(cit).ravel().copy()
    ld = np.ascontiguousarray(np.asarray(ldcompute, dtype=np.uint8).ravel())
    out = np.empty_like(cit)
    lib.ice3o_nucleation(ctypes.byref(table.consts), ctypes.c_long(cit.size), *[_ptr(x) for x in a],
                         ld.ctypes.data_as(ctypes.c_void_p), _ptr(cit), _ptr(out))
    return cit, out


def rrhong_rimltc(table, t, exn, lvfact, lsfact, tht, rrt, rit, ldcompute):
    lib = load()
    a = [_f64(x).ravel() for x in (t, exn, lvfact, lsfact, tht, rrt, rit)]
    ld = np.ascontiguousarray(np.asarray(ldcompute, dtype=np.uint8).ravel())
    o1, o2 = np.empty(a[0].size), np.empty(a[0].size)
    lib.ice3o_rrhong_rimltc(ctypes.byref(table.consts), ctypes.c_long(o1.size), *[_ptr(x) for x in a],
                            ld.ctypes.data_as(ctypes.c_void_p), _ptr(o1), _ptr(o2))
    return o1, o2


def derived_slopes(table, t, rhodref, pres, rv, rr, rs, rg):
    lib = load()
    a = [_f64(x).ravel() for x in (t, rhodref, pres, rv, rr, rs, rg)]
    n = a[0].size
    out = np.empty((9, n))
    lib.ice3o_derived_slopes(ctypes.byref(table.consts), ctypes.c_long(n), *[_ptr(x) for x in a], _ptr(out))
    return dict(zip(("ssi", "ka", "dv", "ai", "cj", "lbdar", "lbdar_rf", "lbdas", "lbdag"), out))


def compute_pdf(table, ldmicro, rhodref, rct, rit, cf, t, sigma_rc):
    lib = load()
    a = [_f64(x).ravel() for x in (rhodref, rct, rit, cf, t, sigma_rc)]
    ld = np.ascontiguousarray(np.asarray(ldmicro, dtype=np.uint8).ravel())
    n = a[0].size
    out = np.empty((9, n))
    lib.ice3o_compute_pdf(ctypes.byref(table.consts), ctypes.c_long(n), ld.ctypes.data_as(ctypes.c_void_p),
                          *[_ptr(x) for x in a], _ptr(out))
    return dict(zip(("hlc_hcf", "hlc_lcf", "hlc_hrc", "hlc_lrc", "hli_hcf", "hli_lcf", "hli_hri", "hli_lri", "rf"),
                    out))


def process_rates(table, inputs: Dict[str, np.ndarray], ldcompute):
    """Hard-pass process rates; inputs keys: t rhodref pres rv rc rr ri rs rg cit ssi ka dv ai cj
    hlc_hcf hlc_hrc hli_hcf hli_hri, optional cf and rainfr (default 1) and
    tht (default t), which the CLFR/PRFR warm processes use."""
    lib = load()
    keys = ("t", "rhodref", "pres", "rv", "rc", "rr", "ri", "rs", "rg", "cit", "ssi", "ka", "dv", "ai", "cj",
            "hlc_hcf", "hlc_hrc", "hli_hcf", "hli_hri", "cf", "rainfr", "tht")
    n = np.asarray(inputs["t"]).size
    inputs = dict(inputs)
    inputs.setdefault("cf", np.ones(n))
    inputs.setdefault("rainfr", np.ones(n))
    inputs.setdefault("tht", inputs["t"])
    inp = np.ascontiguousarray(np.stack([_f64(inputs[k]).ravel() for k in keys]))
    ld = np.ascontiguousarray(np.asarray(ldcompute, dtype=np.uint8).ravel())
    bu, rs, rg = np.empty((len(NBU_NAMES), n)), np.empty((len(RS_NAMES), n)), np.empty((len(RG_NAMES), n))
    lib.ice3o_process_rates(ctypes.byref(table.consts), ctypes.byref(table.luts), ctypes.c_long(n), _ptr(inp),
                            ld.ctypes.data_as(ctypes.c_void_p), _ptr(bu), _ptr(rs), _ptr(rg))
    res = dict(zip(NBU_NAMES, bu))
    res.update({"rs_" + k: v for k, v in zip(RS_NAMES, rs)})
    res.update({"rg_" + k: v for k, v in zip(RG_NAMES, rg)})
    return res


def rainfr_vert(table, prfr, rr, rs, rg):
    lib = load()
    prfr = _f64(prfr).copy()
    nk, nij = prfr.shape
    a = [_f64(x) for x in (rr, rs, rg)]
    lib.ice3o_rainfr_vert(ctypes.byref(table.consts), nij, nk, _ptr(prfr), *[_ptr(x) for x in a])
    return prfr


def physics_step(table, st: Dict[str, np.ndarray], dt: float, max_passes: int = 0, sed_jax: int = 0,
                 out: Optional[Dict[str, np.ndarray]] = None, elapsed: Optional[list] = None):
    """Oracle chained step (ice3o_physics_step); `st` uses the StepFields names.
    `out`: the arrays of a previous call's result, reused (the in-out fields
    are copied in again from `st`), so that repeated steps allocate nothing.
    `elapsed`: a list the wall time of the step itself (the C call) is
    appended to."""
    lib = load()
    keep = {k: _f64(st[k]) for k in STEP_IN}
    nk, nij = keep["pabs"].shape
    f = StepFields()
    for k, v in keep.items():
        setattr(f, k, _ptr(v))
    for k in ("sea", "town"):
        if st.get(k) is not None:
            keep[k] = _f64(st[k])
            setattr(f, k, _ptr(keep[k]))
    if out is None:
        out = {k: _f64(st[k]).copy() for k in STEP_INOUT}
        out.update({k: np.empty((nk, nij)) for k in STEP_OUT3})
        out.update({k: np.empty(nij) for k in STEP_OUT2})
    else:
        for k in STEP_INOUT:
            np.copyto(out[k], st[k])
    for k, v in out.items():
        setattr(f, k, _ptr(v))
    opt = RainIceOptions(-1, -1, -1, max_passes, sed_jax)
    bits = ctypes.c_uint32(0)
    lib.ice3o_physics_step.argtypes = [ctypes.POINTER(Ice3gbConstants), ctypes.POINTER(Ice3gbLuts), ctypes.c_int,
                                       ctypes.c_int, ctypes.c_double, ctypes.POINTER(RainIceOptions),
                                       ctypes.POINTER(StepFields), ctypes.POINTER(ctypes.c_uint32)]
    t0 = time.perf_counter()
    rc = lib.ice3o_physics_step(ctypes.byref(table.consts), ctypes.byref(table.luts), nij, nk, dt, ctypes.byref(opt),
                                ctypes.byref(f), ctypes.byref(bits))
    if elapsed is not None:
        elapsed.append(time.perf_counter() - t0)
    if rc != 0:
        raise RuntimeError(f"oracle physics_step returned {rc}")
    return out, bits.value
