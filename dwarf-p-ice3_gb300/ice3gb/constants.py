"""Constants table: the reference's ``Phyex(program).to_externals()`` dict
packed into the ``Ice3gbConstants`` / ``Ice3gbLuts`` structs of the C ABI.

The table comes either from a live reference ``Phyex`` object or dict (so a
caller of ``IceAdjustJAX(phyex)`` can pass the same object), or from the
JSON snapshot of ``Phyex("AROME").to_externals()`` shipped in ``data/``.

Two flavours exist because the reference's Python tables diverge from the
PHYEX Fortran it was translated from:

``table="jax"``   the Python values unchanged (parity with the reference JAX);
``table="phyex"`` Fortran values for the known divergences:
  * TMINMIX/TMAXMIX swapped back (src/ice3/phyex_common/nebn.py:244-245 vs
    PHYEX-IAL_CY50T1/micro/modd_nebn.F90:178-179);
  * GAMINC_RIM1/2/4 with bound = BOUND_MIN * ZRATE**(j-1) and RIM4 built on
    BG (rain_ice_parameters.py:1105-1156 vs mode_ini_rain_ice.F90:786-790);
  * snow fall speed of the statistical sedimentation: the Python table
    overwrites EXSEDS with DS-BS (= -1.63) and FSEDS with the LNEWCOEFF
    prefactor (rain_ice_parameters.py:725-731), which makes snow fall at
    ~1e16 m/s; PHYEX (LNEWCOEFF = .FALSE.) uses EXSEDS = (BS+DS-CXS)/(BS-CXS)
    and FSEDS = the value the Python table keeps as SEDS
    (mode_ini_rain_ice.F90:533-536, rain_ice_parameters.py:708-722).
"""
from __future__ import annotations

import ctypes
import json
import os
import re
from dataclasses import dataclass
from typing import Any, Dict, List, Mapping, Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_HEADER = os.path.normpath(os.path.join(_HERE, "..", "..", "include", "ice3gb.h"))

NGAMINC, NACCLBDAS, NACCLBDAR, NDRYLBDAG, NDRYLBDAS, NDRYLBDAR = 80, 40, 40, 40, 80, 40
NWETLBDAH, NWETLBDAS, NWETLBDAG, NWETLBDAR = 40, 80, 40, 40


def constant_names(header: str = _HEADER) -> List[str]:
    """Field order of ``Ice3gbConstants``, read from the X-macro list of the
    public header (the library exports the same list through
    ``ice3gb_constant_name``; a test checks both agree)."""
    with open(header) as fh:
        text = fh.read()
    m = re.search(r"#define ICE3GB_CONSTANTS\(X\)(.*?)\n\s*\n", text, re.S)
    if not m:
        raise RuntimeError(f"ICE3GB_CONSTANTS list not found in {header}")
    body = re.sub(r"/\*.*?\*/", "", m.group(1), flags=re.S)
    return re.findall(r"X\((\w+)\)", body)


CONSTANT_NAMES: List[str] = constant_names()


class Ice3gbConstants(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in CONSTANT_NAMES]


class Ice3gbLuts(ctypes.Structure):
    _fields_ = [
        ("gaminc_rim1", ctypes.c_double * NGAMINC),
        ("gaminc_rim2", ctypes.c_double * NGAMINC),
        ("gaminc_rim4", ctypes.c_double * NGAMINC),
        ("ker_raccss", ctypes.c_double * (NACCLBDAS * NACCLBDAR)),
        ("ker_raccs", ctypes.c_double * (NACCLBDAS * NACCLBDAR)),
        ("ker_saccrg", ctypes.c_double * (NACCLBDAR * NACCLBDAS)),
        ("ker_rdryg", ctypes.c_double * (NDRYLBDAG * NDRYLBDAR)),
        ("ker_sdryg", ctypes.c_double * (NDRYLBDAG * NDRYLBDAS)),
        ("ker_sweth", ctypes.c_double * (NWETLBDAH * NWETLBDAS)),
        ("ker_gweth", ctypes.c_double * (NWETLBDAH * NWETLBDAG)),
        ("ker_rweth", ctypes.c_double * (NWETLBDAH * NWETLBDAR)),
    ]


def load_snapshot(program: str = "AROME") -> Dict[str, Any]:
    """Externals dict from the shipped JSON snapshot (arrays as numpy)."""
    path = os.path.join(_HERE, "data", f"phyex_{program.lower()}.json")
    with open(path) as fh:
        raw = json.load(fh)["externals"]
    out: Dict[str, Any] = {}
    for k, v in raw.items():
        if isinstance(v, dict) and "shape" in v:
            out[k] = np.asarray(v["data"], dtype=np.float64).reshape(v["shape"])
        else:
            out[k] = v
    return out


def externals_from(phyex: Any = None, program: str = "AROME") -> Dict[str, Any]:
    """Accept a reference ``Phyex`` object, an externals mapping, or None."""
    if phyex is None:
        return load_snapshot(program)
    if hasattr(phyex, "to_externals"):
        return dict(phyex.to_externals())
    if isinstance(phyex, Mapping):
        return dict(phyex)
    raise TypeError("phyex must be a Phyex object, an externals mapping or None")


def _gaminc_fortran(ext: Mapping[str, Any]):
    """GAMINC_RIM tables as INI_RAIN_ICE builds them (mode_ini_rain_ice.F90:770-790):
    P(a, bound_j) with bound_j = BOUND_MIN * ZRATE**(j-1), the regularised
    lower incomplete gamma function."""
    from scipy.special import gammainc

    bmin, bmax, n = float(ext["GAMINC_BOUND_MIN"]), float(ext["GAMINC_BOUND_MAX"]), int(ext["NGAMINC"])
    zrate = np.exp(np.log(bmax / bmin) / (n - 1))
    bounds = bmin * zrate ** np.arange(n)
    nus, ds, bs, bg, alphas = (float(ext[k]) for k in ("NUS", "DS", "BS", "BG", "ALPHAS"))
    return (gammainc(nus + (2.0 + ds) / alphas, bounds),
            gammainc(nus + bs / alphas, bounds),
            gammainc(nus + bg / alphas, bounds))


@dataclass
class ConstantsTable:
    """Packed constants for one (program, table flavour)."""

    consts: Ice3gbConstants
    luts: Ice3gbLuts
    values: Dict[str, float]
    table: str

    def as_array(self) -> np.ndarray:
        return np.array([self.values[n] for n in CONSTANT_NAMES], dtype=np.float64)


_DEFAULTS = {"OCND2": 0.0}


def _hail_constants(ext: Mapping[str, Any]) -> Dict[str, float]:
    """The hail constants of INI_RAIN_ICE, which the reference's Python
    initialisation leaves out (rain_ice_parameters.py:1094): hailstone
    characteristics (mode_ini_rain_ice.F90:375-392, 436-437), slope and
    sedimentation (:462-463, :547-549), deposition/melting ventilation
    (:633-636) and wet growth (:1226-1291), the switches of
    modd_param_icen.F90 for AROME (LNULLWETH, LWETHPOST, LCONVHG).  The rain,
    snow and graupel distributions are the table's (ALPHAR, NUR, ...), as for
    the other collection constants of the table."""
    from math import exp, gamma, log, sqrt

    def momg(alpha, nu, p):
        return gamma(nu + p / alpha) / gamma(nu)

    f = lambda k: float(ext[k])  # noqa: E731
    pi = f("PI")
    ah, bh, ch, dh, cch, cxh = 470.0, 3.0, 207.0, 0.64, 4.0e4, -1.0
    f0h, f1h, c1h, alphah, nuh = 0.86, 0.28, 0.5, 1.0, 8.0
    cexvt = f("CEXVT")
    # reference density (mode_ini_rain_ice.F90:493-496); LUPDATE_SNOW = XFRMIN(16) > 0 is off
    ze = 0.5 * exp(f("ALPW") - f("BETAW") / 293.15 - f("GAMW") * log(293.15))
    zrv = (f("RD") / f("RV")) * ze / (101325.0 - ze)
    rho00 = 101325.0 * (1.0 + zrv) / (f("RD") + zrv * f("RV")) / 293.15
    rho00_snow = rho00
    v = {"H_RTMIN": 1.0e-15, "CXH": cxh, "DH": dh}
    v["LBEXH"] = 1.0 / (cxh - bh)
    v["LBH"] = (ah * cch * momg(alphah, nuh, bh)) ** (-v["LBEXH"])
    v["EXSEDH"] = (bh + dh - cxh) / (bh - cxh)
    v["FSEDH"] = (ch * ah * cch * momg(alphah, nuh, bh + dh) * (ah * cch * momg(alphah, nuh, bh)) ** (-v["EXSEDH"])
                  * rho00 ** cexvt)
    v["O0DEPH"] = (4.0 * pi) * cch * c1h * f0h * momg(alphah, nuh, 1.0)
    v["O1DEPH"] = (4.0 * pi) * cch * c1h * f1h * sqrt(ch) * momg(alphah, nuh, 0.5 * dh + 1.5)
    v["EX0DEPH"] = cxh - 1.0
    v["EX1DEPH"] = cxh - 0.5 * (dh + 3.0)
    v["COLIH"], v["COLEXIH"] = 0.01, 0.1
    v["FWETH"] = (pi / 4.0) * cch * ch * (rho00 ** cexvt) * momg(alphah, nuh, dh + 2.0)
    v["COLSH"], v["COLEXSH"] = 0.01, 0.1
    v["FSWETH"] = (pi / 4.0) * cch * f("CCS") * f("A_S") * (rho00_snow ** cexvt)     # LNEWCOEFF = .FALSE.
    al_s, nu_s, bs = f("ALPHAS"), f("NUS"), f("BS")
    v["LBSWETH1"] = momg(alphah, nuh, 2.0) * momg(al_s, nu_s, bs)
    v["LBSWETH2"] = 2.0 * momg(alphah, nuh, 1.0) * momg(al_s, nu_s, bs + 1.0)
    v["LBSWETH3"] = momg(al_s, nu_s, bs + 2.0)
    v["COLGH"], v["COLEXGH"] = 0.01, 0.1
    v["FGWETH"] = (pi / 4.0) * cch * f("CCG") * f("AG") * (rho00 ** cexvt)
    al_g, nu_g, bg = f("ALPHAG"), f("NUG"), f("BG")
    v["BG"] = bg
    v["LBGWETH1"] = momg(alphah, nuh, 2.0) * momg(al_g, nu_g, bg)
    v["LBGWETH2"] = 2.0 * momg(alphah, nuh, 1.0) * momg(al_g, nu_g, bg + 1.0)
    v["LBGWETH3"] = momg(al_g, nu_g, bg + 2.0)
    v["FRWETH"] = (pi / 4.0) * cch * f("CCR") * f("AR") * (rho00 ** cexvt)
    al_r, nu_r, br = f("ALPHAR"), f("NUR"), f("BR")
    v["LBRWETH1"] = momg(alphah, nuh, 2.0) * momg(al_r, nu_r, br)
    v["LBRWETH2"] = 2.0 * momg(alphah, nuh, 1.0) * momg(al_r, nu_r, br + 1.0)
    v["LBRWETH3"] = momg(al_r, nu_r, br + 2.0)
    # tabulation grids (:1265-1291): one magnitude of lambda over 10 points
    for x, n, lo, hi in (("S", 80, 2.5e1, 2.5e9), ("G", 40, 1.0e3, 1.0e7), ("R", 40, 1.0e3, 1.0e7),
                         ("H", 40, 1.0e3, 1.0e7)):
        zrate = log(hi / lo) / float(n - 1)
        v[f"NWETLBDA{x}"] = float(n)
        v[f"WETINTP1{x}"] = 1.0 / zrate
        v[f"WETINTP2{x}"] = 1.0 - log(lo) / zrate
    v["LNULLWETH"], v["LWETHPOST"], v["LCONVHG"] = 1.0, 1.0, 1.0
    return v


# XFRMIN_NAM(1:40) of modd_param_icen.F90:366-395 (the Fortran defaults; the
# reference's Python table holds uninitialised values at 9, 22, 30 and 38)
_FRMIN = {1: 0., 2: 0., 3: 0., 4: 0., 5: 0., 6: 0., 7: 1., 8: 1., 9: 1., 10: 10., 11: 1., 12: 0., 13: 1.0e-15,
          14: 120., 15: 1.0e-4, 16: 0., 17: 0., 18: 0., 19: 0., 20: 0., 21: 1., 22: 1., 23: 0.5, 24: 1.5,
          25: 30., 26: 0., 27: 0., 28: 0., 29: 0., 30: 1., 39: 0.25, 40: 0.15}


def _frmin_constants() -> Dict[str, float]:
    return {f"FRMIN{i}": float(_FRMIN.get(i, 0.0)) for i in range(1, 41)}


def _hail_kernels() -> Dict[str, np.ndarray]:
    d = np.load(os.path.join(_HERE, "data", "hail_kernels.npz"))
    return {k: d[k] for k in ("ker_sweth", "ker_gweth", "ker_rweth")}


def build_table(phyex: Any = None, table: str = "jax", program: str = "AROME",
                overrides: Optional[Mapping[str, float]] = None) -> ConstantsTable:
    if table not in ("jax", "phyex"):
        raise ValueError("table must be 'jax' or 'phyex'")
    ext = externals_from(phyex, program)
    hail = {**_hail_constants(ext), **_frmin_constants()}
    values: Dict[str, float] = {}
    for name in CONSTANT_NAMES:
        if name in ext:
            values[name] = float(ext[name])
        elif name in _DEFAULTS:
            values[name] = _DEFAULTS[name]
        elif name in hail:
            values[name] = hail[name]
        else:
            raise KeyError(f"constant {name} missing from the externals table")
    rim1 = np.asarray(ext["GAMINC_RIM1"], dtype=np.float64)
    rim2 = np.asarray(ext["GAMINC_RIM2"], dtype=np.float64)
    rim4 = np.asarray(ext["GAMINC_RIM4"], dtype=np.float64)
    if table == "phyex":
        values["TMINMIX"], values["TMAXMIX"] = 253.16, 273.16
        rim1, rim2, rim4 = _gaminc_fortran(ext)
        bs, ds, cxs = float(ext["BS"]), float(ext["DS"]), float(ext["CXS"])
        values["EXSEDS"] = (bs + ds - cxs) / (bs - cxs)
        values["FSEDS"] = float(ext["SEDS"])
    if overrides:
        for k, v in overrides.items():
            if k not in values:
                raise KeyError(k)
            values[k] = float(v)
    consts = Ice3gbConstants(*[values[n] for n in CONSTANT_NAMES])
    luts = Ice3gbLuts()

    def fill(dst, arr, shape):
        a = np.ascontiguousarray(np.asarray(arr, dtype=np.float64)[: shape[0], : shape[1]]
                                 if len(shape) == 2 else np.asarray(arr, dtype=np.float64)[: shape[0]])
        if a.shape != tuple(shape):
            raise ValueError(f"lookup table has shape {a.shape}, expected {shape}")
        ctypes.memmove(dst, a.ctypes.data, a.nbytes)

    fill(luts.gaminc_rim1, rim1, (NGAMINC,))
    fill(luts.gaminc_rim2, rim2, (NGAMINC,))
    fill(luts.gaminc_rim4, rim4, (NGAMINC,))
    fill(luts.ker_raccss, ext["ker_raccss"], (NACCLBDAS, NACCLBDAR))
    fill(luts.ker_raccs, ext["ker_raccs"], (NACCLBDAS, NACCLBDAR))
    fill(luts.ker_saccrg, ext["ker_saccrg"], (NACCLBDAR, NACCLBDAS))
    fill(luts.ker_rdryg, ext["ker_rdryg"], (NDRYLBDAG, NDRYLBDAR))
    fill(luts.ker_sdryg, ext["ker_sdryg"], (NDRYLBDAG, NDRYLBDAS))
    hk = _hail_kernels()
    fill(luts.ker_sweth, hk["ker_sweth"], (NWETLBDAH, NWETLBDAS))
    fill(luts.ker_gweth, hk["ker_gweth"], (NWETLBDAH, NWETLBDAG))
    fill(luts.ker_rweth, hk["ker_rweth"], (NWETLBDAH, NWETLBDAR))
    return ConstantsTable(consts=consts, luts=luts, values=values, table=table)


def luts_arrays(t: ConstantsTable) -> Dict[str, np.ndarray]:
    """Numpy views of the lookup tables (for tests)."""
    L = t.luts
    return {
        "gaminc_rim1": np.ctypeslib.as_array(L.gaminc_rim1).copy(),
        "gaminc_rim2": np.ctypeslib.as_array(L.gaminc_rim2).copy(),
        "gaminc_rim4": np.ctypeslib.as_array(L.gaminc_rim4).copy(),
        "ker_raccss": np.ctypeslib.as_array(L.ker_raccss).reshape(NACCLBDAS, NACCLBDAR).copy(),
        "ker_raccs": np.ctypeslib.as_array(L.ker_raccs).reshape(NACCLBDAS, NACCLBDAR).copy(),
        "ker_saccrg": np.ctypeslib.as_array(L.ker_saccrg).reshape(NACCLBDAR, NACCLBDAS).copy(),
        "ker_rdryg": np.ctypeslib.as_array(L.ker_rdryg).reshape(NDRYLBDAG, NDRYLBDAR).copy(),
        "ker_sdryg": np.ctypeslib.as_array(L.ker_sdryg).reshape(NDRYLBDAG, NDRYLBDAS).copy(),
    }
