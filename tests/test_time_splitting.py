"""MRSTEP / TSTEP_TS time splitting of the ICE4 sub-stepping
(micro/mode_ice4_stepping.F90:191-197 the outer-iteration budget
INB_ITER_MAX and the sub-step ZTSTEP, :255-259 ZTIME_LASTCALL, :387-397 the
TSTEP_TS limit, :402-453 the MRSTEP limits against Z0RT and ZMAXB).

The reference's Python port has no time splitting (MRSTEP and TSTEP_TS are
only parameters there: ice_parameters.py:430-479) and its Fortran cannot be
compiled here, so the oracle's restatement is pinned by its invariants:
limits that cannot bind leave the step bit for bit unchanged, a TSTEP_TS
sub-step forces at least PTSTEP / TSTEP_TS outer iterations on every active
point, and the water budget closes.  Then the device code's host build (CPU)
and the device kernels (GPU) against the oracle."""
import ctypes

import numpy as np
import pytest

from parity import assert_parity, sensitivity
from test_hail import INPR7, SRC7, _fields, _report_ties, _run_device, _scale, _untie, hail_state, host_libs  # noqa: F401

DT = 50.0
SRC6, INPR6 = SRC7[:-1], INPR7[:-1]


def _table(**kw):
    from ice3gb.constants import build_table
    return build_table(table="phyex", overrides=kw)


def _keys(nrr):
    return (SRC7, INPR7) if nrr == 7 else (SRC6, INPR6)


def _scale_ts(x, ref, fl, k, src):
    """The terms of a source: those of the hail tests, and for a condensed
    species the condensate of the point, which the sub-steps may carry
    through the species and deplete to a rounding residual of it within the
    step (snow converted to graupel in one TSTEP_TS sub-step and melted in
    the next: graupel is zero before and after)."""
    s = _scale(x, ref, fl, k)
    if k in src[1:]:
        s = s + sum(np.abs(x[j]) for j in src[1:])
    return s


# ---------------------------------------------------------------------------- oracle invariants (CPU)

@pytest.mark.parametrize("nrr", [6.0, 7.0])
def test_unbinding_limits_leave_the_step_unchanged(nrr):
    """MRSTEP = 1 kg/kg is never reached within a step and TSTEP_TS = PTSTEP
    gives one sub-step: the splitting must not change a bit."""
    import oracle
    x = hail_state(16 * 16, seed=11)
    base, _ = oracle.rain_ice(_table(NRR=nrr), x, DT)
    for kw in ({"MRSTEP": 1.0}, {"TSTEP_TS": DT}, {"MRSTEP": 1.0, "TSTEP_TS": DT}):
        out, bits = oracle.rain_ice(_table(NRR=nrr, **kw), x, DT)
        assert bits == 0
        for k in base:
            np.testing.assert_array_equal(out[k], base[k], err_msg=f"{kw} {k}")


def _stepping_point_counts(t, x, idx):
    """Outer iterations of ICE4_STEPPING at the given points (oracle hook)."""
    import oracle
    lib = oracle.load()
    names = ("exn", "rhodref", "pabs", "tht", "rvt", "rct", "rrt", "rit", "rst", "rgt", "cit", "ths", "rvs", "rcs",
             "rrs", "ris", "rss", "rgs", "cldfr", "sigs")
    outer = np.zeros(len(idx), dtype=np.int64)
    for j, (k, i) in enumerate(idx):
        inp = np.array([x[n][k, i] for n in names], dtype=np.float64)
        out = np.zeros(10)
        o, inn = ctypes.c_int(), ctypes.c_int()
        lib.ice3o_stepping_point(ctypes.byref(t.consts), ctypes.byref(t.luts), ctypes.c_double(DT), 4096,
                                 inp.ctypes.data_as(ctypes.c_void_p), out.ctypes.data_as(ctypes.c_void_p),
                                 ctypes.byref(o), ctypes.byref(inn))
        assert out[9] == 0.0
        outer[j] = o.value
    return outer


def test_tstep_ts_forces_sub_steps():
    """With TSTEP_TS = 10 s on a 50 s step every point that steps at all
    makes at least five outer iterations (ZTSTEP = 10 s), without it most
    make one; MRSTEP = 5e-6 kg/kg makes more of them than the default."""
    x = hail_state(8 * 8, seed=12)
    rng = np.random.default_rng(0)
    idx = [(int(k), int(i)) for k, i in zip(rng.integers(0, 90, 200), rng.integers(0, 64, 200))]
    base = _stepping_point_counts(_table(), x, idx)
    ts = _stepping_point_counts(_table(TSTEP_TS=10.0), x, idx)
    mr = _stepping_point_counts(_table(MRSTEP=5e-6), x, idx)
    active = base > 0
    assert active.sum() > 100
    assert np.all(ts[active] >= 5) and np.median(base[active]) <= 2
    assert np.all(mr >= base) and np.mean(mr > base) > 0.05


@pytest.mark.parametrize("kw", [{"MRSTEP": 5e-5}, {"TSTEP_TS": 10.0}, {"MRSTEP": 1e-5, "TSTEP_TS": 20.0}])
def test_time_split_water_budget_closes(kw):
    import oracle
    t = _table(NRR=7.0, **kw)
    x = hail_state(16 * 16, seed=13)
    out, bits = oracle.rain_ice(t, x, DT)
    assert bits == 0
    rhodz = x["rhodref"] * x["dzz"]
    col = (rhodz * sum(out[k] - x[k] for k in SRC7)).sum(axis=0) * DT
    precip = sum(out[k] for k in INPR7) * t.values["RHOLW"] * DT
    scale = (rhodz * sum(np.abs(x[k]) for k in SRC7)).sum(axis=0) * DT
    assert np.abs(col + precip).max() <= 1e-12 * scale.max()
    base, _ = oracle.rain_ice(_table(NRR=7.0), x, DT)
    assert np.abs(out["rrs"] - base["rrs"]).max() > 0.0


# ---------------------------------------------------------------------------- host build (CPU)

@pytest.mark.parametrize("nrr,kw", [(6.0, {"MRSTEP": 5e-5}), (6.0, {"TSTEP_TS": 10.0}),
                                    (7.0, {"MRSTEP": 1e-5, "TSTEP_TS": 20.0}),
                                    (6.0, {"MRSTEP": 5e-5, "SUBG_RC_RR_ACCR": 1.0, "SUBG_RR_EVAP": 1.0})])
def test_time_split_host_build_matches_oracle(host_libs, nrr, kw):
    """rain_ice_point's time-splitting instantiation built for the host, then
    the statistical sedimentation after it, against the oracle."""
    import oracle
    t = _table(NRR=nrr, LSEDIM_AFTER=1.0, **kw)
    nij, nk = 16 * 16, 90
    x = hail_state(nij, seed=14)
    src, inpr = _keys(nrr)
    keep, f = _fields(x, nk, nij)
    keys = np.zeros(nij * nk, dtype=np.uint32)
    capped = host_libs["rain_ice_point_host"].rain_ice_points_host_ts(
        ctypes.byref(t.consts), ctypes.byref(t.luts), nij, nk, ctypes.c_double(DT), 4096, ctypes.byref(f),
        keys.ctypes.data_as(ctypes.c_void_p))
    assert capped == 0
    host_libs["sedimentation_host"].sed_stat_rain_ice_host(ctypes.byref(t.consts), nij, nk, ctypes.c_double(DT),
                                                           ctypes.byref(f))
    ref, spread = sensitivity(lambda y: oracle.rain_ice(t, y, DT, max_passes=4096)[0], x, rel=1e-12, trials=4)
    fl, _ = oracle.rain_ice(t, x, DT, max_passes=4096, with_fpr=True, with_ties=True)
    # MRSTEP thresholds on the sub-step are frequent (a species grown from
    # zero to MRSTEP that then depletes), and the sedimentation after the
    # sub-stepping carries them down the column
    spread, share, exempt = _untie(spread, fl["tie"], max_share=0.15)
    for k in ("ths",) + src + ("cit",) + inpr:
        sc = _scale_ts(x, ref, fl, k, src) if k in ("ths",) + src else None
        stats = assert_parity(keep[k], ref[k], spread[k], f"time split host {kw}/{k}", scale=sc,
                              max_frac_conditioned=0.01 + share[k])
        _report_ties(f"time split host {kw}/{k}", keep[k], ref[k], sc, exempt[k], stats)


# ---------------------------------------------------------------------------- GPU

@pytest.mark.gpu
@pytest.mark.parametrize("nrr,kw", [(6.0, {"MRSTEP": 5e-5}), (6.0, {"TSTEP_TS": 10.0}),
                                    (7.0, {"MRSTEP": 1e-5, "TSTEP_TS": 20.0}),
                                    (6.0, {"MRSTEP": 5e-5, "SUBG_RC_RR_ACCR": 1.0, "SUBG_RR_EVAP": 1.0})])
def test_time_split_device_matches_oracle(nrr, kw):
    import oracle
    t = _table(NRR=nrr, **kw)
    x = hail_state(32 * 32, seed=15)
    src, inpr = _keys(nrr)
    ref, spread = sensitivity(lambda y: oracle.rain_ice(t, y, DT)[0], x, rel=1e-12, trials=4)
    fl, _ = oracle.rain_ice(t, x, DT, with_fpr=True, with_ties=True)
    spread, share, exempt = _untie(spread, fl["tie"], sed_after=False)
    got, ri = _run_device(t, x)
    for k in ("ths",) + src + ("cit",) + inpr:
        sc = _scale_ts(x, ref, fl, k, src) if k in ("ths",) + src else None
        stats = assert_parity(got[k], ref[k], spread[k], f"time split device {kw}/{k}", scale=sc,
                              max_frac_conditioned=0.01 + share[k])
        _report_ties(f"time split device {kw}/{k}", got[k], ref[k], sc, exempt[k], stats)
    assert ri.device_status() == 0


@pytest.mark.gpu
def test_unbinding_limits_on_the_device():
    """The time-splitting kernels with limits that cannot bind give the
    default kernels' results bit for bit."""
    x = hail_state(16 * 16, seed=16)
    base, _ = _run_device(_table(), x)
    got, _ = _run_device(_table(MRSTEP=1.0, TSTEP_TS=DT), x)
    for k in base:
        np.testing.assert_array_equal(got[k], base[k], err_msg=k)


@pytest.mark.gpu
def test_physics_step_takes_the_time_splitting():
    """The chained step (ice_adjust -> rain_ice -> ice_adjust) dispatches to
    the time-splitting kernels: limits that cannot bind give the default
    step bit for bit, MRSTEP = 5e-5 another step."""
    from ice3gb.components import Ice3Handle
    from test_gpu_rain_ice import _gpu_step, _np_state, _step_state
    st = _step_state(_np_state(16 * 16, seed=22))
    base = _gpu_step(Ice3Handle(_table()), st)
    same = _gpu_step(Ice3Handle(_table(MRSTEP=1.0, TSTEP_TS=DT)), st)
    for k in base:
        np.testing.assert_array_equal(same[k], base[k], err_msg=k)
    h = Ice3Handle(_table(MRSTEP=5e-5))
    split = _gpu_step(h, st)
    assert h.status() == 0
    assert max(np.abs(split[k] - base[k]).max() for k in ("ths", "rrs", "rss")) > 0.0



# ---------------------------------------------------------------------------- with OCND2

def _ocnd2_device(t, x):
    import torch
    from ice3gb import RainIce
    ri = RainIce()
    ri.table = t
    m = {"exn": "exn", "dzz": "dzz", "rhodref": "rhodref", "exnref": "exnref", "pres": "pabs", "cldfr": "cldfr",
         "sigs": "sigs", "th_t": "tht", "rv_t": "rvt", "rc_t": "rct", "rr_t": "rrt", "ri_t": "rit", "rs_t": "rst",
         "rg_t": "rgt", "ci_t": "cit", "hlc_hrc": "hlc_hrc", "hlc_hcf": "hlc_hcf", "hli_hri": "hli_hri",
         "hli_hcf": "hli_hcf", "ths": "ths", "rvs": "rvs", "rcs": "rcs", "rrs": "rrs", "ris": "ris", "rss": "rss",
         "rgs": "rgs", "sea": "sea", "town": "town", "ssio": "ssio", "ssiu": "ssiu", "ifr": "ifr", "icldfr": "icldfr"}
    state = {k: torch.as_tensor(np.ascontiguousarray(x[v])).cuda() for k, v in m.items()}
    new, diag = ri(state, DT)
    got = {"cit": new["ci_t"].cpu().numpy()}
    for k in SRC6 + ("ths",):
        got[k] = new[k].cpu().numpy()
    for k in INPR6:
        got[k] = diag[k].cpu().numpy()
    return got, ri


def test_ocnd2_time_split_oracle_invariants():
    """OCND2 with the time splitting: unbinding limits change no bit, a
    binding MRSTEP changes the step and the water budget still closes."""
    import oracle
    from test_ocnd2 import ocnd2_rain_ice_state
    x = ocnd2_rain_ice_state(16 * 16, seed=17)
    base, _ = oracle.rain_ice(_table(OCND2=1.0), x, DT)
    same, bits = oracle.rain_ice(_table(OCND2=1.0, MRSTEP=1.0, TSTEP_TS=DT), x, DT)
    assert bits == 0
    for k in base:
        np.testing.assert_array_equal(same[k], base[k], err_msg=k)
    t = _table(OCND2=1.0, MRSTEP=5e-5, TSTEP_TS=10.0)
    out, bits = oracle.rain_ice(t, x, DT)
    assert bits == 0
    rhodz = x["rhodref"] * x["dzz"]
    col = (rhodz * sum(out[k] - x[k] for k in SRC6)).sum(axis=0) * DT
    precip = sum(out[k] for k in INPR6) * t.values["RHOLW"] * DT
    scale = (rhodz * sum(np.abs(x[k]) for k in SRC6)).sum(axis=0) * DT
    assert np.abs(col + precip).max() <= 1e-12 * scale.max()
    assert np.abs(out["rvs"] - base["rvs"]).max() > 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("kw", [{"MRSTEP": 5e-5}, {"TSTEP_TS": 10.0}])
def test_ocnd2_time_split_device_matches_oracle(kw):
    import oracle
    from test_ocnd2 import ocnd2_rain_ice_state
    t = _table(OCND2=1.0, **kw)
    x = ocnd2_rain_ice_state(32 * 32, seed=18)
    ref, spread = sensitivity(lambda y: oracle.rain_ice(t, y, DT)[0], x, rel=1e-12, trials=4)
    fl, _ = oracle.rain_ice(t, x, DT, with_fpr=True, with_ties=True)
    # OCND2 sublimates the ice to a rounding residual at about a fifth of the
    # points; with TSTEP_TS every such reset of cit is followed by hard
    # passes (tie bit 3), 6 % of the points of this state
    spread, share, exempt = _untie(spread, fl["tie"], max_share=0.1, sed_after=False)
    got, ri = _ocnd2_device(t, x)
    for k in ("ths",) + SRC6 + ("cit",) + INPR6:
        sc = _scale_ts(x, ref, fl, k, SRC6) if k in ("ths",) + SRC6 else None
        stats = assert_parity(got[k], ref[k], spread[k], f"ocnd2 time split device {kw}/{k}", scale=sc,
                              max_frac_conditioned=0.01 + share[k])
        _report_ties(f"ocnd2 time split device {kw}/{k}", got[k], ref[k], sc, exempt[k], stats)
    assert ri.device_status() == 0
    # limits that cannot bind: the OCND2 kernel's results bit for bit
    base, _ = _ocnd2_device(_table(OCND2=1.0), x)
    same, _ = _ocnd2_device(_table(OCND2=1.0, MRSTEP=1.0, TSTEP_TS=DT), x)
    for k in base:
        np.testing.assert_array_equal(same[k], base[k], err_msg=k)
