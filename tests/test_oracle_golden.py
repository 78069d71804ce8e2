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
