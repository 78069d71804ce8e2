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
