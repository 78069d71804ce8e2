"""The rain_ice kernel's per-point code (rain_ice_point.cuh, the function the
device runs per lane) built for the host and compared with the oracle on the
CPU: after the oracle's sedimentation, the ICE4 point processing must give
the oracle's sources within the parity criterion.  Catches algorithm changes
in the kernel code without a GPU; the device build differs only by FMA
contraction."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from parity import assert_parity, sensitivity

HERE = os.path.dirname(os.path.abspath(__file__))
DT = 50.0


@pytest.fixture(scope="module")
def host_lib(tmp_path_factory):
    out = tmp_path_factory.mktemp("rip") / "librip_host.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC",
                    "-I", os.path.join(HERE, "..", "include"), os.path.join(HERE, "rain_ice_point_host.cpp"),
                    "-o", str(out)], check=True)
    return ctypes.CDLL(str(out))


@pytest.mark.parametrize("seed", [0, 7])
def test_rain_ice_point_host_build_matches_oracle(host_lib, seed):
    import oracle
    from ice3gb import _abi
    from ice3gb.constants import build_table
    from ice3gb.state import make_state
    from test_gpu_rain_ice import _abi_rain_ice_state

    nij, nk = 32 * 32, 90
    t = build_table(table="phyex")
    st = {k: v.numpy() for k, v in make_state(nij, nk, seed=seed, precip=True).items()}
    abi = _abi_rain_ice_state(st)

    def run_host(x):
        sed = oracle.sedimentation(t, x, DT, True)
        keep, f = {}, _abi.RainIceFields()
        for k in ("exn", "dzz", "rhodref", "exnref", "pabs", "cldfr", "sigs", "tht", "rvt", "rct", "rrt", "rit",
                  "rst", "rgt", "sea", "town"):
            keep[k] = np.ascontiguousarray(x[k], dtype=np.float64)
            setattr(f, k, keep[k].ctypes.data)
        for k in ("cit", "hlc_hrc", "hlc_hcf", "hli_hri", "hli_hcf", "ths", "rvs"):
            keep[k] = np.array(x[k], dtype=np.float64)
            setattr(f, k, keep[k].ctypes.data)
        for k in ("rcs", "rrs", "ris", "rss", "rgs"):
            keep[k] = np.array(sed[k], dtype=np.float64)
            setattr(f, k, keep[k].ctypes.data)
        for k in ("evap3d", "rainfr"):
            keep[k] = np.zeros((nk, nij))
            setattr(f, k, keep[k].ctypes.data)
        keys = np.zeros(nij * nk, dtype=np.uint32)
        capped = host_lib.rain_ice_points_host(ctypes.byref(t.consts), ctypes.byref(t.luts), nij, nk,
                                               ctypes.c_double(DT), 256, ctypes.byref(f),
                                               keys.ctypes.data_as(ctypes.c_void_p))
        assert capped == 0
        return keep

    def run_oracle(x):
        return oracle.rain_ice(t, x, DT)[0]

    got = run_host(abi)
    ref, spread = sensitivity(run_oracle, abi, rel=1e-12, trials=6)
    for k in ("ths", "rvs", "rcs", "rrs", "ris", "rss", "rgs", "cit"):
        scale = np.abs(abi[k]) + np.abs(ref[k]) if k != "cit" else None
        if k in ("rcs", "rrs", "ris", "rss", "rgs"):
            # the sources also carry the sedimentation flux divergence, whose
            # terms are of the size of the flux over rho dz
            fl, _ = oracle.rain_ice(t, abi, DT, with_fpr=True)
            f_ = fl["fpr_" + {"rcs": "c", "rrs": "r", "ris": "i", "rss": "s", "rgs": "g"}[k]]
            fa = np.concatenate([f_[1:], np.zeros_like(f_[:1])], axis=0)
            scale = scale + (np.abs(f_) + np.abs(fa)) / (abi["rhodref"] * abi["dzz"])
        assert_parity(got[k], ref[k], spread[k], f"host rain_ice_point/{k}", scale=scale)


# (SUBG_RC_RR_ACCR, SUBG_RR_EVAP, SUBG_AUCV_RC, SUBG_AUCV_RI); the CLFR
# partition (3 / 1) makes the precipitation fraction take fractional values
SUBG_CASES = [(1, 2, 3, 1), (0, 1, 1, 0), (1, 0, 3, 0), (0, 2, 3, 1)]


@pytest.mark.parametrize("accr,evap,aucv_rc,aucv_ri", SUBG_CASES)
def test_subgrid_warm_options_host_build_matches_oracle(host_lib, accr, evap, aucv_rc, aucv_ri):
    """SUBG_RC_RR_ACCR (NONE 0 / PRFR 1) x SUBG_RR_EVAP (NONE 0 / CLFR 1 /
    PRFR 2): the device code's host build (precipitation fraction per column
    first when a PRFR option is set, then the points) against the oracle's
    RAIN_ICE, sources, ci_t, the precipitation fraction and the partitions
    the PRFR initialisation rewrites."""
    import oracle
    from ice3gb import _abi
    from ice3gb.constants import build_table
    from ice3gb.state import make_state
    from test_gpu_rain_ice import _abi_rain_ice_state

    nij, nk = 24 * 24, 90
    t = build_table(table="phyex", overrides={"SUBG_RC_RR_ACCR": accr, "SUBG_RR_EVAP": evap,
                                              "SUBG_AUCV_RC": aucv_rc, "SUBG_AUCV_RI": aucv_ri})
    st = {k: v.numpy() for k, v in make_state(nij, nk, seed=3, precip=True).items()}
    abi = _abi_rain_ice_state(st)

    def run_host(x):
        sed = oracle.sedimentation(t, x, DT, True)
        keep, f = {}, _abi.RainIceFields()
        for k in ("exn", "dzz", "rhodref", "exnref", "pabs", "cldfr", "sigs", "tht", "rvt", "rct", "rrt", "rit",
                  "rst", "rgt", "sea", "town"):
            keep[k] = np.ascontiguousarray(x[k], dtype=np.float64)
            setattr(f, k, keep[k].ctypes.data)
        for k in ("cit", "hlc_hrc", "hlc_hcf", "hli_hri", "hli_hcf", "ths", "rvs"):
            keep[k] = np.array(x[k], dtype=np.float64)
            setattr(f, k, keep[k].ctypes.data)
        for k in ("rcs", "rrs", "ris", "rss", "rgs"):
            keep[k] = np.array(sed[k], dtype=np.float64)
            setattr(f, k, keep[k].ctypes.data)
        for k in ("evap3d", "rainfr"):
            keep[k] = np.zeros((nk, nij))
            setattr(f, k, keep[k].ctypes.data)
        keys = np.zeros(nij * nk, dtype=np.uint32)
        capped = host_lib.rain_ice_points_host_subg(ctypes.byref(t.consts), ctypes.byref(t.luts), nij, nk,
                                                    ctypes.c_double(DT), 256, ctypes.byref(f),
                                                    keys.ctypes.data_as(ctypes.c_void_p))
        assert capped == 0
        return keep

    def run_oracle(x):
        return oracle.rain_ice(t, x, DT)[0]

    got = run_host(abi)
    ref, spread = sensitivity(run_oracle, abi, rel=1e-12, trials=6)
    fl, _ = oracle.rain_ice(t, abi, DT, with_fpr=True)
    for k in ("ths", "rvs", "rcs", "rrs", "ris", "rss", "rgs", "cit"):
        scale = np.abs(abi[k]) + np.abs(ref[k]) if k != "cit" else None
        if k in ("rcs", "rrs", "ris", "rss", "rgs"):
            f_ = fl["fpr_" + {"rcs": "c", "rrs": "r", "ris": "i", "rss": "s", "rgs": "g"}[k]]
            fa = np.concatenate([f_[1:], np.zeros_like(f_[:1])], axis=0)
            scale = scale + (np.abs(f_) + np.abs(fa)) / (abi["rhodref"] * abi["dzz"])
        assert_parity(got[k], ref[k], spread[k], f"host rain_ice subg {accr}/{evap} {k}", scale=scale)
    for k in ("rainfr", "hlc_hcf", "hlc_hrc", "hli_hcf", "hli_hri"):
        assert_parity(got[k], ref[k], spread[k], f"host rain_ice subg {accr}/{evap} {k}")
    if accr == 1 or evap == 2:
        assert np.count_nonzero((ref["rainfr"] > 0) & (ref["rainfr"] < 1)) > 50
    # the options change the step (evap3d itself is kept only on the points
    # active in the call's last pass, so compare the rain source instead)
    none = oracle.rain_ice(build_table(table="phyex", overrides={"SUBG_AUCV_RC": aucv_rc, "SUBG_AUCV_RI": aucv_ri}),
                           abi, DT)[0]
    assert np.count_nonzero(np.abs(ref["rrs"] - none["rrs"]) > 1e-9 * np.abs(none["rrs"]).max()) > 10
