"""Constants table: snapshot vs the reference's Phyex, table flavours, states."""
import os

import numpy as np
import pytest

from ice3gb.constants import CONSTANT_NAMES, build_table, load_snapshot, luts_arrays

# the reference's src/ directory, when a checkout is at hand
REF_SRC = os.environ.get("ICE3GB_REFERENCE_SRC", "")


def test_snapshot_has_every_constant():
    from ice3gb.constants import _frmin_constants, _hail_constants
    ext = load_snapshot()
    # OCND2 has a default; the hail constants come from INI_RAIN_ICE's
    # formulas, which the reference's Python initialisation leaves out, and
    # XFRMIN from the Fortran namelist defaults
    hail = {**_hail_constants(ext), **_frmin_constants()}
    missing = [n for n in CONSTANT_NAMES if n not in ext and n != "OCND2" and n not in hail]
    assert not missing
    assert all(np.isfinite(v) for v in hail.values())
    t = build_table()
    assert t.values["TSTEP"] if "TSTEP" in t.values else True
    L = luts_arrays(t)
    assert L["ker_sdryg"].shape == (40, 80) and np.all(np.isfinite(L["ker_sdryg"]))
    assert L["ker_raccss"][0, 0] == pytest.approx(7.78513)


@pytest.mark.skipif(not os.path.isdir(REF_SRC), reason="ICE3GB_REFERENCE_SRC names no reference checkout")
def test_snapshot_equals_reference_phyex():
    import sys
    sys.path.insert(0, REF_SRC)
    from ice3.phyex_common.phyex import Phyex
    live = build_table(Phyex("AROME", TSTEP=50.0))
    snap = build_table()
    for n in CONSTANT_NAMES:
        assert live.values[n] == snap.values[n], n
    for k, v in luts_arrays(live).items():
        np.testing.assert_array_equal(v, luts_arrays(snap)[k])


def test_phyex_table_fixes():
    j, p = build_table(table="jax"), build_table(table="phyex")
    assert (j.values["TMINMIX"], j.values["TMAXMIX"]) == (273.16, 253.16)
    assert (p.values["TMINMIX"], p.values["TMAXMIX"]) == (253.16, 273.16)
    lp = luts_arrays(p)
    # P(a, x) increasing from ~0 to 1 over the geometric bounds 0.1 .. 1e7
    for k in ("gaminc_rim1", "gaminc_rim2", "gaminc_rim4"):
        assert np.all(np.diff(lp[k]) >= 0) and lp[k][-1] == pytest.approx(1.0) and lp[k][0] < 0.05


def test_synthetic_state_ranges():
    from ice3gb.state import make_state
    st = make_state(64, 90, seed=3, precip=True)
    p, t = st["pabs"].numpy(), st["t"].numpy()
    assert p.shape == (90, 64)
    assert np.all(p[0] > 98000) and np.all(np.abs(p[-1] - 1000.0) < 1e-6)
    assert np.all(t > 200) and np.all(t < 300)
    assert np.all(st["dzz"].numpy() > 0)
    ri = st["ri"].numpy()
    assert np.all(ri[t >= 268.0] == 0.0)
    for k in ("rc", "ri", "rr", "rs", "rg"):
        v = st[k].numpy()
        assert np.all(v >= 0) and 0.2 < np.mean(v == 0) < 0.9
    np.testing.assert_allclose(st["rvs"].numpy() * 50.0, st["rv"].numpy(), rtol=1e-15)
    again = make_state(64, 90, seed=3, precip=True)
    for k, v in st.items():
        np.testing.assert_array_equal(v.numpy(), again[k].numpy())
