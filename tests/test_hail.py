"""Hail (NRR = 7, the ICE4 scheme with its eighth species): ICE4_FAST_RH
(micro/mode_ice4_fast_rh.F90), the graupel -> hail wet-growth conversion
(mode_ice4_fast_rg.F90:331-351), the hail rows of ICE4_TENDENCIES, the
stepping over eight variables, the hail species of both sedimentation
schemes and of ICE4_CORRECT_NEGATIVITIES.

The reference's JAX port and Python initialisation have no hail
(rain_ice_parameters.py:1094) and its Fortran cannot be compiled here, so the
pins are: the hail kernel tables against the values of the Fortran data
files (the snapshot in ice3gb/data/hail_kernels.npz), and the oracle's
ICE4_FAST_RH against a second, pure-Python restatement of the Fortran.  Then
the device code's host build (CPU) and the device kernels (GPU) against the
oracle, and the water budget of a step."""
import ctypes
import math
import os
import subprocess

import numpy as np
import pytest

from helpers import TOL
from parity import assert_parity, sensitivity

HERE = os.path.dirname(os.path.abspath(__file__))
DT = 50.0
SRC7 = ("rvs", "rcs", "rrs", "ris", "rss", "rgs", "rhs")
INPR7 = ("inprc", "inprr", "inpri", "inprs", "inprg", "inprh")


def _table(**kw):
    from ice3gb.constants import build_table
    return build_table(table="phyex", overrides={"NRR": 7.0, **kw})


def hail_state(nij, seed, nk=90):
    """A rain_ice state (ABI names) with hail: log-normal contents around
    1e-4 kg/kg on 40 % of the points, with a matching source."""
    from ice3gb.state import make_state
    from test_gpu_rain_ice import _abi_rain_ice_state
    st = {k: v.numpy() for k, v in make_state(nij, nk, seed=seed, precip=True).items()}
    x = _abi_rain_ice_state(st)
    rng = np.random.default_rng(seed + 1000)
    rh = np.exp(rng.normal(np.log(1e-4), 1.5, (nk, nij))) * (rng.uniform(size=(nk, nij)) < 0.4)
    x["rht"] = rh
    x["rhs"] = rh / DT * rng.uniform(0.5, 1.5, (nk, nij))
    return x


# ---------------------------------------------------------------------------- tables and constants

def test_hail_kernel_tables_and_grids():
    d = np.load(os.path.join(HERE, "..", "dwarf-p-ice3_gb300", "ice3gb", "data", "hail_kernels.npz"))
    t = _table()
    # entries of the Fortran data statements (mode_read_xker_sweth.F90)
    assert d["ker_sweth"][0, 0] == 0.615237e+01 and d["ker_sweth"][39, 79] == 0.106726e-01
    for name, shape in (("sweth", (40, 80)), ("gweth", (40, 40)), ("rweth", (40, 40))):
        assert d[f"ker_{name}"].shape == shape and np.all(np.isfinite(d[f"ker_{name}"]))
    # the tables reach the library's Ice3gbLuts unchanged
    import ctypes as ct
    buf = np.frombuffer((ct.c_double * (ct.sizeof(t.luts) // 8)).from_buffer_copy(t.luts))
    np.testing.assert_array_equal(buf[9840:13040], d["ker_sweth"].ravel())
    np.testing.assert_array_equal(buf[13040:14640], d["ker_gweth"].ravel())
    np.testing.assert_array_equal(buf[14640:16240], d["ker_rweth"].ravel())
    # the interpolation grids of INI_RAIN_ICE are those the tables were made on
    v = t.values
    for x, tab, key in (("H", "sweth", "H"), ("S", "sweth", "S"), ("G", "gweth", "G"), ("R", "rweth", "R")):
        lo, hi = float(d[f"{tab}_PWETLBDA{key}_MIN"]), float(d[f"{tab}_PWETLBDA{key}_MAX"])
        n = int(d[f"{tab}_KWETLBDA{key}"])
        zrate = math.log(hi / lo) / (n - 1)
        assert v[f"NWETLBDA{x}"] == n
        assert abs(v[f"WETINTP1{x}"] - 1.0 / zrate) <= 1e-15 * abs(v[f"WETINTP1{x}"])
        assert abs(v[f"WETINTP2{x}"] - (1.0 - math.log(lo) / zrate)) <= 1e-14 * abs(v[f"WETINTP2{x}"])
    # hailstone characteristics the tables assume (CH, DH, ALPHAH = 1, NUH = 8)
    assert float(d["sweth_PCH"]) == 207.0 and float(d["sweth_PDH"]) == v["DH"]


# ---------------------------------------------------------------------------- ICE4_FAST_RH pin

def _interp2d(lt, x1, x2, n1, n2, p11, p12, p21, p22):
    """INTERP_MICRO_2D (micro/interp_micro.func.h:126-269), one point, 1-based table."""
    z1 = max(1.00001, min(n1 - 0.00001, p11 * math.log(x1) + p12))
    i1 = int(z1)
    f1 = z1 - i1
    z2 = max(1.00001, min(n2 - 0.00001, p21 * math.log(x2) + p22))
    i2 = int(z2)
    f2 = z2 - i2
    L = lambda a, b: lt[a - 1, b - 1]  # noqa: E731
    return ((L(i1 + 1, i2 + 1) * f2 - L(i1 + 1, i2) * (f2 - 1.0)) * f1
            - (L(i1, i2 + 1) * f2 - L(i1, i2) * (f2 - 1.0)) * (f1 - 1.0))


def fast_rh_py(v, kers, x, ldwetg):
    """mode_ice4_fast_rh.F90 for one point on a hard pass (LDSOFT = .FALSE.,
    LDCOMPUTE, LNEWCOEFF = .FALSE.), with the derived fields and slopes of
    mode_ice4_tendencies.F90:311-317, 389-432, written from the Fortran text
    as plain Python.  Returns (PRH_TEND(1:10), the 12 hail budget terms
    RCWETH .. RHMLTR)."""
    t, rho, p, rv, rc, rr, ri, rs, rg, rh = x
    TT = v["TT"]
    ka = 2.38e-2 + 0.0071e-2 * (t - TT)
    dv = 0.211e-4 * (t / TT) ** 1.94 * (v["P00"] / p)
    cj = v["SCFAC"] * rho ** 0.3 / math.sqrt(1.718e-5 + 0.0049e-5 * (t - TT))
    lbdar = v["LBR"] * (rho * max(rr, v["R_RTMIN"])) ** v["LBEXR"] if rr > 0 else 0.0
    lbdas = min(v["LBDAS_MAX"], v["LBS"] * (rho * max(rs, v["S_RTMIN"])) ** v["LBEXS"]) if rs > 0 else 0.0
    lbdag = v["LBG"] * (rho * max(rg, v["G_RTMIN"])) ** v["LBEXG"] if rg > 0 else 0.0
    lbdah = v["LBH"] * (rho * max(rh, v["H_RTMIN"])) ** v["LBEXH"] if rh > 0 else 0.0
    T = [0.0] * 10   # IRCWETH=1, IRRWETH=2, IRIDRYH=3, IRIWETH=4, IRSDRYH=5, IRSWETH=6, IRGDRYH=7, IRGWETH=8, IFREEZ1=9, IFREEZ2=10
    H = rh > v["H_RTMIN"]
    if H and rc > v["C_RTMIN"]:
        T[0] = lbdah ** (v["CXH"] - v["DH"] - 2.0) * rho ** (-v["CEXVT"])
        T[0] = v["FWETH"] * rc * T[0]
    if H and ri > v["I_RTMIN"]:
        T[3] = lbdah ** (v["CXH"] - v["DH"] - 2.0) * rho ** (-v["CEXVT"])
        T[3] = v["FWETH"] * ri * T[3]
        T[2] = T[3] * (v["COLIH"] * math.exp(v["COLEXIH"] * (t - TT)))
    if H and rs > v["S_RTMIN"]:
        zzw = _interp2d(kers["ker_sweth"], lbdah, lbdas, 40, 80, v["WETINTP1H"], v["WETINTP2H"], v["WETINTP1S"],
                        v["WETINTP2S"])
        T[5] = (v["FSWETH"] * zzw * (lbdas ** (v["CXS"] - v["BS"])) * (lbdah ** v["CXH"])
                * (rho ** (-v["CEXVT"] - 1.0))
                * (v["LBSWETH1"] / (lbdah ** 2) + v["LBSWETH2"] / (lbdah * lbdas) + v["LBSWETH3"] / (lbdas ** 2)))
        T[4] = T[5] * (v["COLSH"] * math.exp(v["COLEXSH"] * (t - TT)))
    if H and rg > v["G_RTMIN"]:
        zzw = _interp2d(kers["ker_gweth"], lbdah, lbdag, 40, 40, v["WETINTP1H"], v["WETINTP2H"], v["WETINTP1G"],
                        v["WETINTP2G"])
        T[7] = (v["FGWETH"] * zzw * (lbdag ** (v["CXG"] - v["BG"])) * (lbdah ** v["CXH"])
                * (rho ** (-v["CEXVT"] - 1.0))
                * (v["LBGWETH1"] / (lbdah ** 2) + v["LBGWETH2"] / (lbdah * lbdag) + v["LBGWETH3"] / (lbdag ** 2)))
        T[6] = T[7]
        if not ldwetg:
            T[6] = T[6] * (v["COLGH"] * math.exp(v["COLEXGH"] * (t - TT)))
    if H and rr > v["R_RTMIN"]:
        zzw = _interp2d(kers["ker_rweth"], lbdah, lbdar, 40, 40, v["WETINTP1H"], v["WETINTP2H"], v["WETINTP1R"],
                        v["WETINTP2R"])
        T[1] = (v["FRWETH"] * zzw * (lbdar ** (-4)) * (lbdah ** v["CXH"]) * (rho ** (-v["CEXVT"] - 1.0))
                * (v["LBRWETH1"] / (lbdah ** 2) + v["LBRWETH2"] / (lbdah * lbdar) + v["LBRWETH3"] / (lbdar ** 2)))
    rdryh_init = T[0] + T[2] + T[4] + T[1] + T[6]
    rweth_init = 0.0
    llweth = lldryh = False
    if H:
        e = rv * p / (v["EPSILO"] + rv)
        if v["LEVLIMIT"]:
            e = min(e, math.exp(v["ALPI"] - v["BETAI"] / t - v["GAMI"] * math.log(t)))
        T[8] = ka * (TT - t) + (dv * (v["LVTT"] + (v["CPV"] - v["CL"]) * (t - TT)) * (v["ESTT"] - e) / (v["RV"] * t))
        T[8] = T[8] * (v["O0DEPH"] * lbdah ** v["EX0DEPH"] + v["O1DEPH"] * cj * lbdah ** v["EX1DEPH"]) / \
            (rho * (v["LMTT"] - v["CL"] * (TT - t)))
        T[9] = (rho * (v["LMTT"] + (v["CI"] - v["CL"]) * (TT - t))) / (rho * (v["LMTT"] - v["CL"] * (TT - t)))
        rweth_init = max(T[3] + T[5] + T[7], max(0.0, T[8] + T[9] * (T[3] + T[5] + T[7])))
        llweth = max(0.0, rweth_init - T[3] - T[5] - T[7]) <= max(0.0, rdryh_init - T[2] - T[4] - T[6])
        llweth = llweth and (rdryh_init > 0.0 if v["LNULLWETH"] else rweth_init > 0.0)
        if not v["LWETHPOST"]:
            llweth = llweth and t < TT
        lldryh = (t < TT and rdryh_init > 1.e-20
                  and max(0.0, rweth_init - T[3] - T[5]) > max(0.0, rdryh_init - T[2] - T[4]))
    rdryhg = rdryh_init * rweth_init / (rdryh_init + rweth_init) if (v["LCONVHG"] and lldryh) else 0.0
    wet = [T[0], T[3], T[5], T[7], rweth_init - T[3] - T[5] - T[7] - T[0]] if llweth else [0.0] * 5
    dry = [T[0], T[2], T[4], T[1], T[6], rdryhg] if lldryh else [0.0] * 6
    mlt = 0.0
    if H and t > TT:
        e = rv * p / (v["EPSILO"] + rv)
        if v["LEVLIMIT"]:
            e = min(e, math.exp(v["ALPW"] - v["BETAW"] / t - v["GAMW"] * math.log(t)))
        mlt = ka * (TT - t) + dv * (v["LVTT"] + (v["CPV"] - v["CL"]) * (t - TT)) * (v["ESTT"] - e) / (v["RV"] * t)
        mlt = max(0.0, (-mlt * (v["O0DEPH"] * lbdah ** v["EX0DEPH"] + v["O1DEPH"] * cj * lbdah ** v["EX1DEPH"])
                        - (T[0] + T[1]) * (rho * v["CL"] * (TT - t))) / (rho * v["LMTT"]))
    return T, wet + dry + [mlt]


def test_oracle_fast_rh_matches_python_restatement():
    import oracle
    t = _table()
    v = {k: float(x) for k, x in t.values.items()}
    kers = np.load(os.path.join(HERE, "..", "dwarf-p-ice3_gb300", "ice3gb", "data", "hail_kernels.npz"))
    rng = np.random.default_rng(5)
    n = 600
    T = rng.uniform(240.0, 285.0, n)
    rho = rng.uniform(0.4, 1.2, n)
    p = rho * 287.0 * T
    mix = lambda pz: np.exp(rng.uniform(np.log(1e-7), np.log(5e-3), n)) * (rng.uniform(size=n) > pz)  # noqa: E731
    rv = rng.uniform(0.5, 1.1, n) * 0.622 * 611.0 * np.exp(17.5 * (T - 273.15) / (T - 36.0)) / p
    x = np.stack([T, rho, p, rv, mix(0.3), mix(0.3), mix(0.3), mix(0.3), mix(0.3), mix(0.1)], axis=1)
    ldwetg = (rng.uniform(size=n) < 0.5).astype(np.uint8)
    out = np.empty((n, 24))
    lib = oracle.load()
    lib.ice3o_fast_rh(ctypes.byref(t.consts), ctypes.byref(t.luts), ctypes.c_long(n),
                      np.ascontiguousarray(x).ctypes.data_as(ctypes.c_void_p), ldwetg.ctypes.data_as(ctypes.c_void_p),
                      out.ctypes.data_as(ctypes.c_void_p))
    active = np.zeros(12, dtype=int)
    for i in range(n):
        tend, bud = fast_rh_py(v, kers, tuple(x[i]), bool(ldwetg[i]))
        ref = np.array(tend + bud)
        got = np.concatenate([out[i, :10], out[i, 12:24]])
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-300, err_msg=f"point {i}")
        active += np.array(bud) != 0.0
    # every branch taken: wet and dry growth terms, hail -> graupel, melting
    assert np.all(active > 5), active


# ---------------------------------------------------------------------------- host build and budget (CPU)

@pytest.fixture(scope="module")
def host_libs(tmp_path_factory):
    d = tmp_path_factory.mktemp("hail")
    libs = {}
    for name in ("rain_ice_point_host", "sedimentation_host"):
        out = d / f"lib{name}.so"
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-I",
                        os.path.join(HERE, "..", "include"), os.path.join(HERE, f"{name}.cpp"), "-o", str(out)],
                       check=True)
        libs[name] = ctypes.CDLL(str(out))
    return libs


def _fields(x, nk, nij):
    from ice3gb import _abi
    keep, f = {}, _abi.RainIceFields()
    for k in ("exn", "dzz", "rhodref", "exnref", "pabs", "cldfr", "sigs", "tht", "rvt", "rct", "rrt", "rit", "rst",
              "rgt", "rht", "sea", "town"):
        keep[k] = np.ascontiguousarray(x[k], dtype=np.float64)
        setattr(f, k, keep[k].ctypes.data)
    for k in ("cit", "hlc_hrc", "hlc_hcf", "hli_hri", "hli_hcf", "ths") + SRC7:
        keep[k] = np.array(x[k], dtype=np.float64)
        setattr(f, k, keep[k].ctypes.data)
    for k in ("evap3d", "rainfr"):
        keep[k] = np.zeros((nk, nij))
        setattr(f, k, keep[k].ctypes.data)
    for k in INPR7:
        keep[k] = np.zeros(nij)
        setattr(f, k, keep[k].ctypes.data)
    return keep, f


def _untie(spread, tie, max_share=0.02, sed_after=True):
    """Points where the oracle took a decision on rounding residuals
    (ice3o_rain_ice_ties) get an unbounded allowance.  Bit 0, a graupel or
    hail growth-mode choice (the wet-growth estimate minus what it collects,
    a difference of several non-zero rates that is zero up to rounding,
    against the dry-growth one): the point, for every field, and when the
    sedimentation follows the sub-stepping (sed_after) also the levels below
    it, where the sedimentation carries the outcome, and the surface fields
    of its column.  Bit 2, an MRSTEP threshold on the sub-step already
    chosen (a soft pass or a new outer iteration), and bit 3, a hard pass
    of a later outer iteration after a bit-1 reset, the same.  Bit 1, the
    reset of the ice concentration after a pass that left the ice at a
    rounding residual: cit at the point.  They must stay a small share of
    the grid."""
    nk = tie.shape[0]
    growth = (tie & 13) != 0
    if sed_after:
        below = np.flip(np.maximum.accumulate(np.flip(growth, axis=0), axis=0), axis=0)   # tie at or above k
        cols = below[0]
    else:
        below, cols = growth, np.zeros(tie.shape[1], dtype=bool)
    cit_tie = (tie & 2) != 0
    assert below.mean() <= max_share, f"{below.mean():.2%} of the points lie at or below a growth-mode tie"
    # ice sublimating to zero within a pass is common (OCND2 states: up to a
    # fifth of the points); only cit is exempted there
    assert cit_tie.mean() <= 0.3, f"{cit_tie.mean():.2%} of the points reset cit on an ice residual"
    out, share, exempt = {}, {}, {}
    for k, v in spread.items():
        v = np.array(v, dtype=np.float64)
        share[k] = 0.0
        exempt[k] = np.zeros(v.shape, dtype=bool)
        if v.ndim == 2 and v.shape[0] == nk:
            m = below | cit_tie if k == "cit" else below
            v[m] = np.inf
            share[k] = float(m.mean())
            exempt[k] = m
        elif v.ndim == 1 and v.shape[0] == cols.shape[0]:
            v[cols] = np.inf
            share[k] = float(cols.mean())
            exempt[k] = cols
        out[k] = v
    return out, share, exempt


def _report_ties(name, got, ref, scale, exempt, stats, tol=1e-10, max_other=1e-3):
    """How the tie allowance was used: of the exempt points (a tie and, with
    the sedimentation after it, the levels below), how many differ from the
    oracle beyond the 1e-10 bound, and by how much at most; the other points
    may need the conditioning spread on at most `max_other` of the grid."""
    got, ref = np.asarray(got, dtype=np.float64), np.asarray(ref, dtype=np.float64)
    fin = np.isfinite(ref)
    rms = float(np.sqrt(np.mean(ref[fin] ** 2))) if fin.any() else 0.0
    mag = np.abs(ref) if scale is None else np.maximum(np.abs(ref), np.asarray(scale, dtype=np.float64))
    d = np.where(fin, np.abs(got - ref), 0.0)
    over = d > tol * np.maximum(mag, 1e-5 * rms)
    used = over & exempt
    worst = float(np.max(d[used] / np.maximum(mag[used], 1e-5 * rms + 1e-300))) if used.any() else 0.0
    other = int(stats["n_spread"]) - int(used.sum())
    print(f"{name}: exempt {int(exempt.sum())}, of which beyond 1e-10 {int(used.sum())} (worst rel {worst:.2e}); "
          f"other points needing the spread {other} of {stats['n']}")
    assert other <= max_other * stats["n"], f"{name}: {other} points outside the ties needed the spread"


def _scale(x, ref, fl, k):
    rhodz = x["rhodref"] * x["dzz"]
    s = np.abs(x[k]) + np.abs(ref[k])
    key = {"rcs": "c", "rrs": "r", "ris": "i", "rss": "s", "rgs": "g", "rhs": "h"}.get(k)
    if key:
        f_ = fl["fpr_" + key]
        fa = np.concatenate([f_[1:], np.zeros_like(f_[:1])], axis=0)
        s = s + (np.abs(f_) + np.abs(fa)) / rhodz
    return s


def test_hail_host_build_matches_oracle(host_libs):
    """rain_ice_point's hail instantiation and the hail sweep, built for the
    host: the points, then the statistical sedimentation (LSEDIM_AFTER),
    against the oracle's RAIN_ICE."""
    import oracle
    t = _table(LSEDIM_AFTER=1.0, LDEPOSC=0.0)
    nij, nk = 24 * 24, 90
    x = hail_state(nij, seed=3)

    keep, f = _fields(x, nk, nij)
    keys = np.zeros(nij * nk, dtype=np.uint32)
    capped = host_libs["rain_ice_point_host"].rain_ice_points_host_hail(
        ctypes.byref(t.consts), ctypes.byref(t.luts), nij, nk, ctypes.c_double(DT), 256, ctypes.byref(f),
        keys.ctypes.data_as(ctypes.c_void_p))
    assert capped == 0
    host_libs["sedimentation_host"].sed_stat_rain_ice_host(ctypes.byref(t.consts), nij, nk, ctypes.c_double(DT),
                                                           ctypes.byref(f))
    ref, spread = sensitivity(lambda y: oracle.rain_ice(t, y, DT)[0], x, rel=1e-12, trials=4)
    fl, _ = oracle.rain_ice(t, x, DT, with_fpr=True, with_ties=True)
    spread, share, exempt = _untie(spread, fl["tie"])
    for k in ("ths",) + SRC7 + ("cit",) + INPR7:
        sc = _scale(x, ref, fl, k) if k in ("ths",) + SRC7 else None
        stats = assert_parity(keep[k], ref[k], spread[k], f"hail host/{k}", scale=sc,
                              max_frac_conditioned=0.01 + share[k])
        _report_ties(f"hail host/{k}", keep[k], ref[k], sc, exempt[k], stats)
    assert np.count_nonzero(ref["inprh"]) > 50


@pytest.mark.parametrize("sedim", [1.0, 0.0])      # STAT, SPLI
def test_hail_water_budget_closes(sedim):
    import oracle
    t = _table(SEDIM=sedim)
    nij, nk = 16 * 16, 90
    x = hail_state(nij, seed=4)
    out, bits = oracle.rain_ice(t, x, DT)
    assert bits == 0
    rhodz = x["rhodref"] * x["dzz"]
    d = sum(out[k] - x[k] for k in SRC7)
    col = (rhodz * d).sum(axis=0) * DT
    precip = sum(out[k] for k in INPR7) * t.values["RHOLW"] * DT
    scale = (rhodz * sum(np.abs(x[k]) for k in SRC7)).sum(axis=0) * DT
    assert np.abs(col + precip).max() <= 1e-12 * scale.max()
    assert np.count_nonzero(out["inprh"]) > 20
    # the hail changes the other species (conversion, collection, melting)
    o6, _ = oracle.rain_ice(_table(SEDIM=sedim, NRR=6.0), x, DT)
    assert np.abs(out["rgs"] - o6["rgs"]).max() > 0.0


# ---------------------------------------------------------------------------- GPU

def _run_device(t, x, host=False, **kw):
    import torch
    from ice3gb import RainIce
    ri = RainIce()
    ri.table = t
    m = {"exn": "exn", "dzz": "dzz", "rhodref": "rhodref", "exnref": "exnref", "pres": "pabs", "cldfr": "cldfr",
         "sigs": "sigs", "th_t": "tht", "rv_t": "rvt", "rc_t": "rct", "rr_t": "rrt", "ri_t": "rit", "rs_t": "rst",
         "rg_t": "rgt", "rh_t": "rht", "ci_t": "cit", "hlc_hrc": "hlc_hrc", "hlc_hcf": "hlc_hcf",
         "hli_hri": "hli_hri", "hli_hcf": "hli_hcf", "ths": "ths", "rvs": "rvs", "rcs": "rcs", "rrs": "rrs",
         "ris": "ris", "rss": "rss", "rgs": "rgs", "rhs": "rhs", "sea": "sea", "town": "town"}
    state = {k: (np.ascontiguousarray(x[v]) if host else torch.as_tensor(np.ascontiguousarray(x[v])).cuda())
             for k, v in m.items()}
    new, diag = ri(state, DT, **kw)
    res = {}
    back = {"ci_t": "cit", "ths": "ths", "rvs": "rvs", "rcs": "rcs", "rrs": "rrs", "ris": "ris", "rss": "rss",
            "rgs": "rgs", "rhs": "rhs"}
    # without hail (NRR = 6) there is no rhs / inprh
    for k, v in back.items():
        if k in new:
            res[v] = np.asarray(new[k] if host else new[k].cpu().numpy())
    for k in INPR7:
        if k in diag:
            res[k] = np.asarray(diag[k] if host else diag[k].cpu().numpy())
    return res, ri


@pytest.mark.gpu
@pytest.mark.parametrize("sedim,after", [(1.0, False), (1.0, True), (0.0, False)])
def test_hail_device_matches_oracle(sedim, after):
    import oracle
    t = _table(SEDIM=sedim)
    nij = 32 * 32
    x = hail_state(nij, seed=5)
    ref, spread = sensitivity(lambda y: oracle.rain_ice(t, y, DT, lsedim_after=int(after))[0], x, rel=1e-12,
                              trials=4)
    fl, _ = oracle.rain_ice(t, x, DT, lsedim_after=int(after), with_fpr=True, with_ties=True)
    spread, share, exempt = _untie(spread, fl["tie"])
    got, ri = _run_device(t, x, lsedim_after=after)
    for k in ("ths",) + SRC7 + ("cit",) + INPR7:
        sc = _scale(x, ref, fl, k) if k in ("ths",) + SRC7 else None
        stats = assert_parity(got[k], ref[k], spread[k], f"hail device/{k}", scale=sc,
                              max_frac_conditioned=0.01 + share[k])
        _report_ties(f"hail device/{k}", got[k], ref[k], sc, exempt[k], stats)
    assert ri.device_status() == 0
    assert np.count_nonzero(got["inprh"]) > 50


@pytest.mark.gpu
def test_hail_host_entry_point_equals_device():
    t = _table()
    x = hail_state(20 * 20, seed=6)
    dev, _ = _run_device(t, x)
    host, _ = _run_device(t, x, host=True)
    for k in dev:
        np.testing.assert_array_equal(host[k], dev[k], err_msg=k)
    assert TOL > 0


# ---------------------------------------------------------------------------- hail with OCND2

def ocnd2_hail_state(nij, seed):
    """An OCND2 rain_ice state (the ice_adjust OCND2 outputs included) with
    hail on 40 % of the points."""
    from test_ocnd2 import ocnd2_rain_ice_state
    x = ocnd2_rain_ice_state(nij, seed)
    nk = x["exn"].shape[0]
    rng = np.random.default_rng(seed + 2000)
    rh = np.exp(rng.normal(np.log(1e-4), 1.5, (nk, nij))) * (rng.uniform(size=(nk, nij)) < 0.4)
    x["rht"] = rh
    x["rhs"] = rh / DT * rng.uniform(0.5, 1.5, (nk, nij))
    return x


def test_ocnd2_hail_water_budget_closes():
    """OCND2 with hail (the LOCND2 rows and LLMICRO with PRHT,
    rain_ice.F90:349-356): the water budget of the step closes."""
    import oracle
    t = _table(OCND2=1.0)
    x = ocnd2_hail_state(16 * 16, seed=7)
    out, bits = oracle.rain_ice(t, x, DT)
    assert bits == 0
    rhodz = x["rhodref"] * x["dzz"]
    col = (rhodz * sum(out[k] - x[k] for k in SRC7)).sum(axis=0) * DT
    precip = sum(out[k] for k in INPR7) * t.values["RHOLW"] * DT
    scale = (rhodz * sum(np.abs(x[k]) for k in SRC7)).sum(axis=0) * DT
    assert np.abs(col + precip).max() <= 1e-12 * scale.max()
    assert np.count_nonzero(out["inprh"]) > 20


@pytest.mark.gpu
@pytest.mark.parametrize("kw", [{}, {"MRSTEP": 5e-5}])
def test_ocnd2_hail_device_matches_oracle(kw):
    import oracle
    import torch
    from ice3gb import RainIce
    t = _table(OCND2=1.0, **kw)
    x = ocnd2_hail_state(32 * 32, seed=8)
    ref, spread = sensitivity(lambda y: oracle.rain_ice(t, y, DT)[0], x, rel=1e-12, trials=4)
    fl, _ = oracle.rain_ice(t, x, DT, with_fpr=True, with_ties=True)
    spread, share, exempt = _untie(spread, fl["tie"], max_share=0.1, sed_after=False)
    ri = RainIce()
    ri.table = t
    m = {"exn": "exn", "dzz": "dzz", "rhodref": "rhodref", "exnref": "exnref", "pres": "pabs", "cldfr": "cldfr",
         "sigs": "sigs", "th_t": "tht", "rv_t": "rvt", "rc_t": "rct", "rr_t": "rrt", "ri_t": "rit", "rs_t": "rst",
         "rg_t": "rgt", "rh_t": "rht", "ci_t": "cit", "hlc_hrc": "hlc_hrc", "hlc_hcf": "hlc_hcf",
         "hli_hri": "hli_hri", "hli_hcf": "hli_hcf", "ths": "ths", "rvs": "rvs", "rcs": "rcs", "rrs": "rrs",
         "ris": "ris", "rss": "rss", "rgs": "rgs", "rhs": "rhs", "sea": "sea", "town": "town", "ssio": "ssio",
         "ssiu": "ssiu", "ifr": "ifr", "icldfr": "icldfr"}
    state = {k: torch.as_tensor(np.ascontiguousarray(x[v])).cuda() for k, v in m.items()}
    new, diag = ri(state, DT)
    got = {"cit": new["ci_t"].cpu().numpy()}
    for k in ("ths",) + SRC7:
        got[k] = new[k].cpu().numpy()
    for k in INPR7:
        got[k] = diag[k].cpu().numpy()
    for k in ("ths",) + SRC7 + ("cit",) + INPR7:
        sc = _scale(x, ref, fl, k) if k in ("ths",) + SRC7 else None
        stats = assert_parity(got[k], ref[k], spread[k], f"ocnd2 hail device {kw}/{k}", scale=sc,
                              max_frac_conditioned=0.01 + share[k])
        _report_ties(f"ocnd2 hail device {kw}/{k}", got[k], ref[k], sc, exempt[k], stats)
    assert ri.device_status() == 0
    assert np.count_nonzero(got["inprh"]) > 50
