"""Pin the CPU oracle against the golden vectors made by running the
reference's own JAX code (tests/golden/make_golden.py).  No GPU needed."""
import numpy as np
import pytest

from conftest import load_golden, rel_err
from helpers import TOL

import oracle
from ice3gb.constants import build_table

DT = 50.0


@pytest.fixture(scope="module")
def jax_table():
    return build_table(table="jax")


IA_OUT = ("t", "rv_out", "rc_out", "ri_out", "cldfr", "hlc_hrc", "hlc_hcf", "hli_hri", "hli_hcf", "cph", "lv",
          "ls", "rvs", "rcs", "ris", "ths")


@pytest.mark.parametrize("case", ["ia_std", "ia_mf"])
def test_ice_adjust_matches_reference_jax(jax_table, case):
    g = load_golden(case)
    st = {k[3:]: v for k, v in g.items() if k.startswith("in_")}
    out = oracle.ice_adjust(jax_table, st, DT)
    for name in IA_OUT:
        err = rel_err(out[name], g[f"out_{name}"])
        assert err <= TOL, f"{case}/{name}: rel err {err:.3e}"


def test_ice_adjust_conserves_total_water(jax_table):
    # reference test: tests/components/test_ice_adjust_jax.py:268-283
    g = load_golden("ia_std")
    st = {k[3:]: v for k, v in g.items() if k.startswith("in_")}
    out = oracle.ice_adjust(jax_table, st, DT)
    before = st["rv"] + st["rc"] + st["ri"]
    after = out["rv_out"] + out["rc_out"] + out["ri_out"]
    assert np.max(np.abs(after - before) / before) < 1e-14


def test_sedimentation_matches_reference_jax(jax_table):
    g = load_golden("sed_jax")
    st = {k[3:]: v for k, v in g.items() if k.startswith("in_")}
    out = oracle.sedimentation(jax_table, st, DT, fortran=False, with_fpr=True)
    for name in ("rcs", "rrs", "ris", "rss", "rgs", "fpr_c", "fpr_r", "fpr_i", "fpr_s", "fpr_g", "inprc", "inprr",
                 "inpri", "inprs", "inprg"):
        err = rel_err(out[name], g[f"out_{name}"])
        assert err <= TOL, f"{name}: rel err {err:.3e}"


def _proc_inputs():
    g = load_golden("processes")
    inp = {k[3:]: v for k, v in g.items() if k.startswith("in_")}
    out = {k[4:]: v for k, v in g.items() if k.startswith("out_")}
    return g, inp, out


def test_nucleation_rrhong_rimltc(jax_table):
    g, i, o = _proc_inputs()
    ld = i["ld"] > 0.5
    cit, rvheni = oracle.nucleation(jax_table, i["tht"], i["pres"], i["rhodref"], i["exn"], i["lsfact"], i["t"],
                                    i["rv"], i["cit"], ld)
    assert rel_err(cit, o["nucl_cit"]) <= TOL
    assert rel_err(rvheni, o["nucl_rvheni"]) <= TOL
    rrhong, rimltc = oracle.rrhong_rimltc(jax_table, i["t"], i["exn"], i["lvfact"], i["lsfact"], i["tht"],
                                          i["rr"], i["ri"], ld)
    assert rel_err(rrhong, o["rrhong"]) <= TOL
    assert rel_err(rimltc, o["rimltc"]) <= TOL


def test_derived_fields_and_slopes(jax_table):
    g, i, o = _proc_inputs()
    d = oracle.derived_slopes(jax_table, i["t"], i["rhodref"], i["pres"], i["rv"], i["rr"], i["rs"], i["rg"])
    for k in ("ssi", "ka", "dv", "ai", "cj", "lbdar", "lbdar_rf", "lbdas", "lbdag"):
        assert rel_err(d[k], o[k]) <= TOL, k


@pytest.mark.parametrize("tag,aucv_rc,aucv_ri", [("pdf_sigm", 1, 0), ("none", 0, 0), ("clfr", 3, 1)])
def test_compute_pdf(tag, aucv_rc, aucv_ri):
    # table enum (ice_parameters.py:42-47): NONE=0 PDF=1 ADJU=2 CLFR=3; the JAX
    # stencil numbers them 0=NONE 1=CLFR 2=ADJU 3=PDF (ice4_compute_pdf.py:42-44)
    table = build_table(table="jax", overrides={"SUBG_AUCV_RC": aucv_rc, "SUBG_AUCV_RI": aucv_ri,
                                                "SUBG_PR_PDF": 0})
    g, i, o = _proc_inputs()
    r = oracle.compute_pdf(table, i["ld"] > 0.5, i["rhodref"], i["rc"], i["ri"], i["cf"], i["t"], i["sigma_rc"])
    for k in ("hlc_hcf", "hlc_lcf", "hlc_hrc", "hlc_lrc", "hli_hcf", "hli_lcf", "hli_hri", "hli_lri", "rf"):
        assert rel_err(r[k], o[f"pdf_{tag}_{k}"]) <= TOL, f"{tag}/{k}"


def test_slow_warm_fast_processes(jax_table):
    g, i, o = _proc_inputs()
    ld = i["ld"] > 0.5
    d = oracle.derived_slopes(jax_table, i["t"], i["rhodref"], i["pres"], i["rv"], i["rr"], i["rs"], i["rg"])
    inp = dict(t=i["t"], rhodref=i["rhodref"], pres=i["pres"], rv=i["rv"], rc=i["rc"], rr=i["rr"], ri=i["ri"],
               rs=i["rs"], rg=i["rg"], cit=i["cit"], ssi=d["ssi"], ka=d["ka"], dv=d["dv"], ai=d["ai"],
               cj=d["cj"], hlc_hcf=i["hlc_hcf"], hlc_hrc=i["hlc_hrc"], hli_hcf=i["hli_hcf"],
               hli_hri=i["hli_hri"])
    r = oracle.process_rates(jax_table, inp, ld)
    for k in ("rchoni", "rvdeps", "riaggs", "riauts", "rvdepg", "rcautr", "rcaccr", "rrevav", "rcberi",
              "ricfrrg", "rrcfrig", "ricfrr"):
        assert rel_err(r[k], o[k]) <= TOL, k
    for k in ("rcdryg", "ridryg", "riwetg"):
        assert rel_err(r["rg_" + k], o["rg_" + k]) <= TOL, k
    assert rel_err(r["rs_freez1"], o["rs_freez1"]) <= TOL
    assert rel_err(r["rs_freez2"], o["rs_freez2"]) <= TOL
    # melting of snow/graupel pinned on the points without riming/accretion inputs
    m = ld & (i["rc"] == 0) & (i["rr"] == 0)
    assert rel_err(np.where(m, r["rsmltg"], 0.0), o["rsmltg"]) <= TOL
    m = ld & (i["rr"] == 0)
    assert rel_err(np.where(m, r["rgmltr"], 0.0), o["rgmltr"]) <= TOL


def test_rainfr_vert(jax_table):
    g = load_golden("processes")
    out = oracle.rainfr_vert(jax_table, g["rf_in_prfr"], g["rf_in_rr"], g["rf_in_rs"], g["rf_in_rg"])
    assert rel_err(out, g["rf_out_prfr"]) <= TOL


@pytest.mark.parametrize("mode", [1, 2])
def test_warm_subgrid_evaporation(mode):
    """CLFR (1) and PRFR (2) rain evaporation (and autoconversion /
    accretion on the same points) against the reference JAX ice4_warm."""
    g = load_golden("warm_subg")
    i = {k[3:]: v for k, v in g.items() if k.startswith("in_")}
    table = build_table(table="jax", overrides={"SUBG_RR_EVAP": mode})
    n = i["t"].size
    z = np.zeros(n)
    inp = dict(t=i["t"], rhodref=i["rhodref"], pres=i["pres"], rv=i["rv"], rc=i["rc"], rr=i["rr"], ri=z, rs=z,
               rg=z, cit=z, ssi=i["ssi"], ka=i["ka"], dv=i["dv"], ai=i["ai"], cj=i["cj"], hlc_hcf=i["hlc_hcf"],
               hlc_hrc=i["hlc_hrc"], hli_hcf=z, hli_hri=z, cf=i["cf"], rainfr=i["rf"], tht=i["tht"])
    r = oracle.process_rates(table, inp, i["ld"] > 0.5)
    for k in ("rcautr", "rcaccr", "rrevav"):
        assert rel_err(r[k], g[f"out{mode}_{k}"]) <= TOL, (mode, k)
    assert np.count_nonzero(g[f"out{mode}_rrevav"]) > 50


# ---- RAIN_ICE / ICE4_STEPPING pieces (tests/golden/ri_pieces.npz) ----------

def _c(a, dtype=np.float64):
    return np.ascontiguousarray(a, dtype=dtype)


def _p(a):
    import ctypes
    return a.ctypes.data_as(ctypes.c_void_p)


@pytest.fixture(scope="module")
def pieces():
    return load_golden("ri_pieces")


def test_rain_ice_thermo_and_mask_match_reference_jax(jax_table, pieces):
    """rain_ice_thermo / rain_ice_mask (src/ice3/jax/stencils/rain_ice.py:95, :141)."""
    import ctypes
    g = pieces
    lib = oracle.load()
    n = g["th_th"].size
    t = _c(g["th_th"] * g["th_exn"])
    ls, lv, micro = np.empty(n), np.empty(n), np.empty(n, dtype=np.uint8)
    lib.ice3o_rain_ice_thermo(ctypes.byref(jax_table.consts), ctypes.c_long(n), _p(t),
                              *(_p(_c(g[f"th_{k}"])) for k in ("rv", "rc", "rr", "ri", "rs", "rg")),
                              _p(ls), _p(lv), _p(micro))
    assert rel_err(ls, g["th_out_ls"]) <= TOL and rel_err(lv, g["th_out_lv"]) <= TOL
    np.testing.assert_array_equal(micro.astype(np.float64), g["th_out_mask"])
    assert 0 < micro.sum() < n


def test_total_tendencies_match_reference_jax(pieces):
    """rain_ice_total_tendencies (src/ice3/jax/stencils/rain_ice.py:19): the
    sources after the sub-stepping, with RVHENI; tolerance relative to the
    terms summed (start source + change over the step)."""
    import ctypes
    g = pieces
    lib = oracle.load()
    names = ("th", "v", "c", "r", "i", "s", "g")
    n = g["tt_rvheni"].size
    r0 = {"th": g["th_th"], "v": g["th_rv"], "c": g["th_rc"], "r": g["th_rr"], "i": g["th_ri"], "s": g["th_rs"],
          "g": g["th_rg"]}
    vend = _c(np.stack([g[f"tt_wr_{k}"] for k in names]))
    r0a = _c(np.stack([r0[k] for k in names]))
    src = _c(np.stack([g[f"tt_src_{k}"] for k in names]))
    lib.ice3o_total_tendencies(ctypes.c_long(n), ctypes.c_double(DT), _p(vend), _p(r0a), _p(_c(g["tt_lvx"])),
                               _p(_c(g["tt_lsx"])), _p(_c(g["tt_rvheni"])), _p(src))
    for i, k in enumerate(names):
        ref = g[f"tt_out_{k}"]
        scale = np.abs(g[f"tt_src_{k}"]) + np.abs(vend[i] - r0a[i]) / DT * (3000.0 if k == "th" else 1.0) \
            + np.abs(g["tt_rvheni"]) * (3000.0 if k == "th" else 1.0)
        assert np.all(np.abs(src[i] - ref) <= TOL * np.maximum(np.abs(ref), scale)), k


def test_fog_deposition_matches_reference_jax(jax_table, pieces):
    """fog_deposition (src/ice3/jax/stencils/rain_ice.py:323)."""
    import ctypes
    g = pieces
    lib = oracle.load()
    n = g["fog_rcs"].size
    rcs, inprc = _c(g["fog_rcs"]).copy(), _c(g["fog_inprc"]).copy()
    lib.ice3o_fog_deposition(ctypes.byref(jax_table.consts), ctypes.c_long(n), _p(_c(g["fog_rct"])),
                             _p(_c(g["fog_rho"])), _p(_c(g["fog_dzz"])), _p(rcs), _p(inprc))
    assert rel_err(rcs, g["fog_out_rcs"]) <= TOL and rel_err(inprc, g["fog_out_inprc"]) <= TOL


def test_aggregation_matches_reference_jax(pieces):
    """ice4_total_tendencies_update (src/ice3/jax/stencils/ice4_tendencies.py:330):
    the oracle's ICE4_TENDENCIES aggregation on the same rates; tolerance
    relative to the sum of the magnitudes of the terms."""
    import ctypes
    g = pieces
    lib = oracle.load()
    n = g["ag_ls"].size
    bu = np.zeros((len(oracle.NBU_NAMES), n))
    mags = {k: np.zeros(n) for k in ("th", "v", "c", "r", "i", "s", "g")}
    for k, v in g.items():
        if k.startswith("ag_") and not k.startswith("ag_out_") and k not in ("ag_ls", "ag_lv"):
            bu[oracle.NBU_NAMES.index(k[3:])] = v
            for m in mags:
                mags[m] += np.abs(v) * (g["ag_ls"] if m == "th" else 1.0)
    A = np.empty((7, n))
    lib.ice3o_aggregate(ctypes.c_long(n), _p(_c(bu)), _p(_c(g["ag_ls"])), _p(_c(g["ag_lv"])), _p(A))
    for i, k in enumerate(("th", "v", "c", "r", "i", "s", "g")):
        ref = g[f"ag_out_{k}"]
        assert np.all(np.abs(A[i] - ref) <= TOL * np.maximum(np.abs(ref), mags[k])), k
        assert np.count_nonzero(ref) > n // 2


def test_step_limiter_matches_reference_jax(jax_table, pieces):
    """ice4_step_limiter (src/ice3/jax/stencils/ice4_stepping.py:109) against
    the oracle's LFEEDBACKT and depletion limits (mode_ice4_stepping.F90:
    284-311) on inputs where their definitions coincide (see make_golden)."""
    import ctypes
    g = pieces
    lib = oracle.load()
    n = g["sl_th"].size
    sp = ("c", "r", "i", "s", "g")
    vart = _c(np.stack([g["sl_th"], np.full(n, 1e-2)] + [g[f"sl_r{k}"] for k in sp]))
    A = _c(np.stack([g["sl_a_th"], np.zeros(n)] + [g[f"sl_a{k}"] for k in sp]))
    B = _c(np.stack([g["sl_b_th"], np.zeros(n)] + [g[f"sl_b{k}"] for k in sp]))
    rsmin = _c(np.zeros(7))
    mt, ld = np.empty(n), np.empty(n, dtype=np.uint8)
    lib.ice3o_step_limiter(ctypes.byref(jax_table.consts), ctypes.c_long(n), ctypes.c_double(DT), _p(rsmin),
                           _p(_c(g["sl_exn"])), _p(vart), _p(A), _p(B), _p(_c(g["sl_t_micro"])),
                           _p(_c(g["sl_ld"], np.uint8)), _p(mt), _p(ld))
    assert rel_err(mt, g["sl_out_dt"]) <= TOL
    np.testing.assert_array_equal(ld.astype(np.float64), g["sl_out_ld"])
    # the inputs exercise every limit: time left, 0 C crossing, depletion, end of step
    left = np.where(g["sl_ld"] > 0, DT - g["sl_t_micro"], 0.0)
    assert np.count_nonzero(mt == 0.0) >= 5 and np.count_nonzero((mt > 0) & (mt < left)) > 100


def test_state_update_matches_reference_jax(pieces):
    """state_update (src/ice3/jax/stencils/ice4_stepping.py:232): x + A dt + B
    and the ice concentration reset where the ice is gone."""
    import ctypes
    g = pieces
    lib = oracle.load()
    n = g["sl_th"].size
    sp = ("c", "r", "i", "s", "g")
    vart = _c(np.stack([g["sl_th"], np.full(n, 1e-2)] + [g[f"su_r{k}"] for k in sp]))
    A = _c(np.stack([g["sl_a_th"], np.zeros(n)] + [g[f"sl_a{k}"] for k in sp]))
    B = _c(np.stack([g["sl_b_th"], np.zeros(n)] + [-np.abs(g[f"sl_b{k}"]) for k in sp]))
    cit = _c(g["su_ci"]).copy()
    lib.ice3o_state_update(ctypes.c_long(n), _p(A), _p(B), _p(_c(g["sl_out_dt"])), _p(_c(g["sl_ld"], np.uint8)),
                           _p(vart), _p(cit))
    for i, k in zip((0, 2, 3, 4, 5, 6), ("th", "c", "r", "i", "s", "g")):
        assert rel_err(vart[i], g[f"su_out_{k}"]) <= TOL, k
    np.testing.assert_array_equal(cit, g["su_out_ci"])
    assert np.count_nonzero((cit == 0) & (g["su_ci"] > 0)) > 10


@pytest.mark.parametrize("case", ["A", "B"])
def test_correct_negativities_matches_reference_jax(jax_table, pieces, case):
    """ice4_correct_negativities (src/ice3/jax/stencils/ice4_correct_negativities.py:14).
    Case A (vapour far above every threshold): the oracle's Fortran form
    (the one rain_ice runs) equals the JAX stencil.  Case B (vapour near
    zero): the JAX form of the vapour refill (snow and graupel up to their
    own minima), which the oracle keeps beside the Fortran one."""
    import ctypes
    g = pieces
    lib = oracle.load()
    v = jax_table.values
    n = g["cn_lsx"].size
    names = ("th", "rv", "rc", "rr", "ri", "rs", "rg")
    x = _c(np.stack([g[f"cn{case}_{k}"] for k in names]))
    fortran = 1 if case == "A" else 0
    smin, gmin = (v["V_RTMIN"], v["V_RTMIN"]) if fortran else (v["S_RTMIN"], v["G_RTMIN"])
    lib.ice3o_correct_negativities(ctypes.c_long(n), fortran, ctypes.c_double(smin), ctypes.c_double(gmin),
                                   _p(_c(g["cn_lvx"])), _p(_c(g["cn_lsx"])), _p(x))
    for i, k in enumerate(names):
        ref = g[f"cn{case}_out_{k}"]
        scale = np.abs(g[f"cn{case}_{k}"]) + (np.abs(x[i] - g[f"cn{case}_{k}"]) if k != "th" else 0.0)
        assert np.all(np.abs(x[i] - ref) <= TOL * np.maximum(np.abs(ref), scale) + 1e-300), k
    assert np.all(x[2:] >= 0.0)


def test_ice_adjust_reference_test_states(jax_table):
    """The states of the reference's own ice_adjust tests
    (tests/components/test_ice_adjust_jax.py: simple_test_data, realistic_test_data,
    the supersaturated state of test_cloud_formation), timestep 60 s: the
    oracle against IceAdjustJAX run on them (tests/golden/ia_fixtures.npz)."""
    g = load_golden("ia_fixtures")
    for case in ("simple", "realistic", "cloud_formation"):
        st = {k[len(case) + 4:]: v for k, v in g.items() if k.startswith(f"{case}_in_")}
        shape = st["pabs"].shape
        flat = {k: np.ascontiguousarray(v.reshape(-1, shape[-1]).T) for k, v in st.items()}   # [nz][nx*ny]
        out = oracle.ice_adjust(jax_table, flat, 60.0)
        for name in IA_OUT:
            ref = g[f"{case}_out_{name}"].reshape(-1, shape[-1]).T
            err = rel_err(out[name], ref)
            assert err <= TOL, f"{case}/{name}: rel err {err:.3e}"
