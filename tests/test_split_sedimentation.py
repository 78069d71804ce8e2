"""Time-split sedimentation (SEDIM = SPLI, mode_ice4_sedimentation_split.F90
followed by ICE4_CORRECT_NEGATIVITIES): the device code's host build against
the oracle, and the column water budget of both (CPU).  The full rain_ice
step with SPLI on the device is checked against the oracle in
tests/test_gpu_rain_ice.py."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from helpers import TOL

HERE = os.path.dirname(os.path.abspath(__file__))
DT = 50.0
SRC = ("rcs", "rrs", "ris", "rss", "rgs")
INPR = ("inprc", "inprr", "inpri", "inprs", "inprg")


@pytest.fixture(scope="module")
def sed_lib(tmp_path_factory):
    out = tmp_path_factory.mktemp("sed") / "libsed_host.so"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", "-I",
                    os.path.join(HERE, "..", "include"), os.path.join(HERE, "sedimentation_host.cpp"), "-o",
                    str(out)], check=True)
    return ctypes.CDLL(str(out))


def _fields(x, nij, nk, sea_town):
    from ice3gb import _abi
    keep, f = {}, _abi.RainIceFields()
    for k in ("exn", "dzz", "rhodref", "exnref", "pabs", "cldfr", "sigs", "tht", "rvt", "rct", "rrt", "rit", "rst",
              "rgt"):
        keep[k] = np.ascontiguousarray(x[k], dtype=np.float64)
        setattr(f, k, keep[k].ctypes.data)
    for k in ("ths", "rvs") + SRC:
        keep[k] = np.array(x[k], dtype=np.float64)
        setattr(f, k, keep[k].ctypes.data)
    for k in ("fpr_c", "fpr_r", "fpr_i", "fpr_s", "fpr_g"):
        keep[k] = np.zeros((nk, nij))
        setattr(f, k, keep[k].ctypes.data)
    for k in INPR:
        keep[k] = np.zeros(nij)
        setattr(f, k, keep[k].ctypes.data)
    if sea_town:
        rng = np.random.default_rng(3)
        keep["sea"] = rng.uniform(0, 1, nij)
        keep["town"] = rng.uniform(0, 0.3, nij)
        f.sea, f.town = keep["sea"].ctypes.data, keep["town"].ctypes.data
    return keep, f


def _state(nij, seed):
    from ice3gb.state import make_state
    from test_gpu_rain_ice import _abi_rain_ice_state
    st = {k: v.numpy() for k, v in make_state(nij, 90, seed=seed, precip=True).items()}
    return _abi_rain_ice_state(st)


def _run(sed_lib, table, x, nij, nk, sea_town, which):
    import oracle
    keep, f = _fields(x, nij, nk, sea_town)
    if which == "host":
        scratch = np.empty(2 * nij * nk)
        ok = sed_lib.sed_split_host(ctypes.byref(table.consts), nij, nk, ctypes.c_double(DT), ctypes.byref(f),
                                    scratch.ctypes.data_as(ctypes.c_void_p))
    else:
        lib = oracle.load()
        ok = lib.ice3o_sedimentation_split(ctypes.byref(table.consts), nij, nk, ctypes.c_double(DT), ctypes.byref(f))
    assert ok == 1
    return keep


@pytest.mark.parametrize("sea_town,lsedic", [(False, 1.0), (True, 1.0), (True, 0.0)])
def test_split_host_build_matches_oracle_and_conserves_water(sed_lib, sea_town, lsedic):
    from ice3gb.constants import build_table
    t = build_table(table="phyex", overrides={"SEDIM": 0.0, "LSEDIC": lsedic})
    nij, nk = 24 * 24, 90
    x = _state(nij, seed=41)
    got = _run(sed_lib, t, x, nij, nk, sea_town, "host")
    ref = _run(sed_lib, t, x, nij, nk, sea_town, "oracle")
    # relative to each field's largest magnitude: the sources are sums of many
    # sub-step changes that cancel at the upper levels
    for k in ("ths", "rvs") + SRC + INPR + ("fpr_r", "fpr_s", "fpr_g"):
        assert np.abs(got[k] - ref[k]).max() <= TOL * np.abs(ref[k]).max() + 1e-300, k
    # sedimentation moves water down and out through the surface; the
    # negativity correction only exchanges it with vapour
    rhodz = x["rhodref"] * x["dzz"]
    for out in (got, ref):
        d = sum(out[k] - x[k] for k in ("rvs",) + SRC)
        col = (rhodz * d).sum(axis=0) * DT
        precip = sum(out[k] for k in INPR) * t.values["RHOLW"] * DT
        scale = (rhodz * sum(np.abs(x[k]) for k in SRC)).sum(axis=0) * DT + 1e-30
        assert np.all(np.abs(col + precip) <= 1e-12 * scale)
    assert (ref["inprr"] > 0).sum() > 100
    if lsedic == 0.0:
        np.testing.assert_array_equal(ref["inprc"], 0.0)
