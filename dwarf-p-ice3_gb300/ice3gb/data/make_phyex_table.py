"""Snapshot the reference's constants table into ``phyex_<program>.json``.

Runs the reference's own ``Phyex(program).to_externals()``
(src/ice3/phyex_common/phyex.py:307-344 of maurinl26/dwarf-p-ice3) and stores
every scalar and every lookup table it returns, so that machines without the
reference checkout (and without its scipy-based initialisation) get the
identical table.  TSTEP/INV_TSTEP are stored but the library always uses the
time step passed at call time.

Usage:  python make_phyex_table.py [--reference-src DIR] [--program AROME]
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference-src", default=os.environ.get("ICE3GB_REFERENCE_SRC"),
                    required="ICE3GB_REFERENCE_SRC" not in os.environ,
                    help="the reference's src/ directory (or set ICE3GB_REFERENCE_SRC)")
    ap.add_argument("--program", default="AROME")
    ap.add_argument("--out", default=None)
    args = ap.parse_args()
    sys.path.insert(0, args.reference_src)
    from ice3.phyex_common.phyex import Phyex  # noqa: E402

    ext = Phyex(args.program, TSTEP=50.0).to_externals()
    table = {}
    for key, val in ext.items():
        if isinstance(val, str):
            table[key] = val
        elif isinstance(val, (bool, int, float, np.integer, np.floating)):
            table[key] = float(val)
        elif isinstance(val, np.ndarray):
            arr = np.asarray(val, dtype=np.float64)
            # np.empty padding rows of the 41-sized reference arrays may hold
            # garbage; they are never read (Fortran indices start at 1).
            if not np.all(np.isfinite(arr)):
                arr = np.where(np.isfinite(arr), arr, 0.0)
            table[key] = {"shape": list(arr.shape), "data": arr.ravel().tolist()}
        elif isinstance(val, (list, tuple)):
            table[key] = [float(v) for v in val]
        else:
            raise TypeError(f"unsupported externals entry {key}: {type(val)}")
    out = args.out or os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                   f"phyex_{args.program.lower()}.json")
    with open(out, "w") as fh:
        json.dump({"program": args.program, "source": "Phyex.to_externals()",
                   "externals": table}, fh, indent=0, sort_keys=True)
    print(f"wrote {out} ({len(table)} entries)")


if __name__ == "__main__":
    main()
