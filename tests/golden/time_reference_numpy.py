"""Time the reference's own IceAdjustJAX, run unmodified in float64 through
the numpy stand-in for jax (refshim.py), on the 64 x 64 x 90 ice_adjust
workload (seed 0, dt = 50 s): the "reference code, numpy backend" CPU
baseline.  One process, numpy's own threading; best of 5 after one warm-up.
The same workload through the C oracle (all host cores) is timed beside it.

Usage:  python tests/golden/time_reference_numpy.py [--reference-src DIR]
(or ICE3GB_REFERENCE_SRC); prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [HERE, os.path.join(REPO, "dwarf-p-ice3_gb300"), os.path.join(REPO, "oracle")]

ARGS = ("sigqsat", "pabs", "sigs", "th", "exn", "exn_ref", "rho_dry_ref", "rv", "rc", "ri", "rr", "rs", "rg",
        "cf_mf", "rc_mf", "ri_mf", "rvs", "rcs", "ris", "ths")


def best_of(fn, n=5):
    fn()
    ts = []
    for _ in range(n):
        t0 = time.perf_counter()
        fn()
        ts.append(time.perf_counter() - t0)
    return min(ts)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference-src", default=os.environ.get("ICE3GB_REFERENCE_SRC"),
                    required="ICE3GB_REFERENCE_SRC" not in os.environ)
    ap.add_argument("--nij", type=int, default=64 * 64)
    args = ap.parse_args()
    import refshim
    refshim.install()
    sys.path.insert(0, args.reference_src)
    np.seterr(all="ignore")
    from ice3.jax.ice_adjust import IceAdjustJAX
    from ice3.phyex_common.phyex import Phyex

    import oracle
    from ice3gb.constants import build_table
    from ice3gb.state import make_state

    dt = 50.0
    st = {k: v.numpy() for k, v in make_state(args.nij, 90, seed=0).items()}
    nk, nij = st["pabs"].shape
    st["sigqsat"] = np.broadcast_to(st["sigqsat"][None, :], (nk, nij)).copy()
    ia = IceAdjustJAX(Phyex("AROME", TSTEP=dt), jit=False)
    x = {k: np.asarray(st[k]).view(refshim.ShimArray) for k in ARGS}
    t_ref = best_of(lambda: ia(**x, timestep=dt))
    table = build_table(table="jax")
    t_orc = best_of(lambda: oracle.ice_adjust(table, {k: st[k] for k in ARGS}, dt))
    n = nk * nij
    print(json.dumps({"workload": f"ice_adjust {nij} columns x {nk} levels ({n} points), FP64, dt={dt}s",
                      "reference_numpy": {"value": n / t_ref, "unit": "grid-points/s", "seconds": t_ref,
                                          "what": "IceAdjustJAX run unmodified through the numpy stand-in",
                                          "processes": 1},
                      "oracle": {"value": n / t_orc, "unit": "grid-points/s", "seconds": t_orc,
                                 "threads": os.cpu_count()},
                      "cpu": os.cpu_count()}))


if __name__ == "__main__":
    main()
