"""Snapshot PHYEX's tabulated hail collection kernels into ``hail_kernels.npz``.

INI_RAIN_ICE reads XKER_SWETH, XKER_GWETH and XKER_RWETH (the normalised
snow / graupel / rain collection kernels of the hailstones, tabulated against
the slope parameters) from the data statements of
PHYEX-IAL_CY50T1/micro/mode_read_xker_sweth.F90, mode_read_xker_gweth.F90 and
mode_read_xker_rweth.F90 of maurinl26/dwarf-p-ice3 (mode_ini_rain_ice.F90:
1300-1470).  The reference's Python initialisation has no hail, so this
script parses those values (and the grid parameters each file states)
and stores them, with the arrays laid out (lbdah, lbda_x) as Ice3gbLuts
holds them.

Usage:  python make_hail_kernels.py [--micro DIR]
"""
from __future__ import annotations

import argparse
import os
import re

import numpy as np

TABLES = {"sweth": (40, 80), "gweth": (40, 40), "rweth": (40, 40)}


def parse(path: str, name: str, shape):
    text = open(path).read()
    arr = np.full(shape, np.nan)
    pat = re.compile(r"PKER_%s\(\s*(\d+)\s*,\s*(\d+)\s*\)\s*=\s*([-+0-9.Ee]+)" % name.upper())
    for i, j, v in pat.findall(text):
        arr[int(i) - 1, int(j) - 1] = float(v)
    if np.isnan(arr).any():
        raise ValueError(f"{path}: {int(np.isnan(arr).sum())} entries of PKER_{name.upper()} missing")
    params = {}
    for key, v in re.findall(r"^\s*(P[A-Z_]+|K[A-Z_]+)\s*=\s*([-+0-9.Ee]+)\s*$", text, re.M):
        params[key] = float(v)
    return arr, params


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--micro", required=True, help="the reference's PHYEX-IAL_CY50T1/micro directory")
    ap.add_argument("--out", default=os.path.join(os.path.dirname(os.path.abspath(__file__)), "hail_kernels.npz"))
    args = ap.parse_args()
    out = {}
    for name, shape in TABLES.items():
        arr, params = parse(os.path.join(args.micro, f"mode_read_xker_{name}.F90"), name, shape)
        out[f"ker_{name}"] = arr
        for k, v in params.items():
            out[f"{name}_{k}"] = np.float64(v)
    np.savez_compressed(args.out, **out)
    print(f"wrote {args.out}: " + ", ".join(f"{k}{v.shape}" for k, v in out.items() if k.startswith("ker_")))


if __name__ == "__main__":
    main()
