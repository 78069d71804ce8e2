"""Standalone drivers of the ICE3 components on the GB300 kernels: the
``ice-adjust`` and ``rain-ice`` commands of the reference's
``standalone-model`` CLI (src/drivers/cli.py:29, :203) with an ``ice3gb``
backend, its field comparison (``compare_fields``, src/drivers/core.py:83-178)
and its tracking file (``write_performance_tracking``, core.py:41-66).

    python -m ice3gb.drivers ice-adjust --dataset ice_adjust.nc \\
        --output-path ice_adjust_run.nc --tracking-file ice_adjust_run.json
    python -m ice3gb.drivers rain-ice --dataset rain_ice.nc ...
    python -m ice3gb.drivers rain-ice --domain 64 1024 90 --seed 0   # synthetic state

Datasets use the PHYEX testprogs layout the reference's tests read
(tests/components/test_ice_adjust_jax.py:455-548,
tests/components/test_rain_ice_jax.py:45-130): 3-D fields
(ngpblks, nflevg, nproma) named PPABSM, PEXNREF, PRHODREF, PTHT, PTHS, PSIGS,
...; species stacks ZRS (ngpblks, krr1, nflevg, nproma; theta first) and
PRT / PRS / PRS_OUT (ngpblks, krr, nflevg, nproma; vapour first); reference
outputs PRS_OUT, PTHS, PCLDFR_OUT, PHLC_HCF_OUT, ...  They are read and
written as netCDF-3 (scipy.io); a netCDF-4 (HDF5) file needs the netCDF4 or
h5py package, which this environment does not have: convert it with
``nccopy -k classic``.  Without a dataset the drivers run a seeded synthetic
AROME-like state (ice3gb.state.make_state) of the given domain and report
timings only.

The run's fields are written with dims (ngpblks, nproma, nflevg) under the
component's state names, as the reference's drivers write them.
"""
from __future__ import annotations

import argparse
import json
import logging
import sys
import time
from typing import Dict, List, Optional, Tuple

import numpy as np

log = logging.getLogger(__name__)

# run field -> reference variable (src/drivers/core.py:104-128)
KEYS_ICE_ADJUST = [("hli_hcf", "PHLI_HCF_OUT"), ("hli_hri", "PHLI_HRI_OUT"), ("hlc_hcf", "PHLC_HCF_OUT"),
                   ("hlc_hrc", "PHLC_HRC_OUT"), ("cldfr", "PCLDFR_OUT"), ("ths", "PTHS"), ("rvs", "PRS_OUT"),
                   ("rcs", "PRS_OUT"), ("ris", "PRS_OUT")]
KEYS_RAIN_ICE = [("rainfr", "ZRAINFR_OUT"), ("fpr", "PFPR_OUT"), ("indep", "ZINDEP_OUT"), ("inprg", "PINPRG_OUT"),
                 ("inprs", "PINPRS_OUT"), ("evap3d", "PEVAP_OUT"), ("inprr", "PINPRR_OUT"),
                 ("inprc", "ZINPRC_OUT"), ("rvs", "PRS_OUT"), ("rcs", "PRS_OUT"), ("rrs", "PRS_OUT"),
                 ("ris", "PRS_OUT"), ("rss", "PRS_OUT"), ("rgs", "PRS_OUT"), ("ci_t", "PCIT_OUT")]
TENDENCIES = ["ths", "rvs", "rcs", "rrs", "ris", "rss", "rgs"]


# ---------------------------------------------------------------------------- netCDF-3 I/O

class DatasetError(RuntimeError):
    pass


def _open(path: str):
    from scipy.io import netcdf_file
    try:
        return netcdf_file(path, "r", mmap=False)
    except (TypeError, ValueError) as e:
        with open(path, "rb") as fh:
            magic = fh.read(4)
        if magic == b"\x89HDF":
            raise DatasetError(f"{path} is netCDF-4 (HDF5): reading it needs netCDF4 or h5py, absent here; "
                               "convert it with `nccopy -k classic`") from e
        raise DatasetError(f"{path}: not a netCDF-3 file ({e})") from e


class NetCDFReader:
    """Fields of a netCDF-3 dataset in the drivers' layout (ngpblks, nproma,
    nflevg) / (ngpblks, krr, nproma, nflevg), as the reference's reader
    returns them (src/drivers/core.py:13-39)."""

    def __init__(self, path: str):
        self.path = path
        self.f = _open(path)
        self.sizes = dict(self.f.dimensions)

    def __contains__(self, name: str) -> bool:
        return name in self.f.variables

    def get_field(self, name: str) -> np.ndarray:
        if name not in self.f.variables:
            raise KeyError(f"variable {name} not found in {self.path}")
        v = self.f.variables[name]
        a = np.array(v[:], dtype=np.float64)
        dims = list(v.dimensions)
        if a.ndim == 3 and "nproma" in dims and "nflevg" in dims and "ngpblks" in dims:
            return np.transpose(a, [dims.index(d) for d in ("ngpblks", "nproma", "nflevg")]).copy()
        if a.ndim == 4 and "nproma" in dims and "nflevg" in dims:
            sp = next((d for d in dims if d not in ("ngpblks", "nproma", "nflevg")), None)
            return np.transpose(a, [dims.index(d) for d in ("ngpblks", sp, "nproma", "nflevg")]).copy()
        return a

    def close(self):
        self.f.close()


def write_dataset(fields: Dict[str, np.ndarray], output_path: str) -> None:
    """Write the run's fields (netCDF-3): 3-D (ngpblks, nproma, nflevg), 2-D
    (ngpblks, nproma), 4-D (ngpblks, <name>_sp, nproma, nflevg)."""
    from scipy.io import netcdf_file
    shapes = [np.shape(v) for v in fields.values() if np.ndim(v) == 3]
    if not shapes:
        raise ValueError("no 3-D field to write")
    g, p, z = shapes[0]
    with netcdf_file(output_path, "w") as f:
        f.createDimension("ngpblks", g)
        f.createDimension("nproma", p)
        f.createDimension("nflevg", z)
        for k, v in fields.items():
            v = np.asarray(v, dtype=np.float64)
            if v.shape == (g, p, z):
                dims = ("ngpblks", "nproma", "nflevg")
            elif v.shape == (g, p):
                dims = ("ngpblks", "nproma")
            elif v.ndim == 4 and v.shape[0] == g and v.shape[2:] == (p, z):
                f.createDimension(f"{k}_sp", v.shape[1])
                dims = ("ngpblks", f"{k}_sp", "nproma", "nflevg")
            else:
                log.debug("skipping %s of shape %s", k, v.shape)
                continue
            var = f.createVariable(k, "d", dims)
            var[:] = v


# ---------------------------------------------------------------------------- metrics / tracking

def field_metrics(ref: np.ndarray, run: np.ndarray) -> Dict[str, float]:
    """The reference's per-field metrics (src/drivers/core.py:97-98, :158-175)."""
    e_inf = float(np.max(np.abs(ref - run)))
    e_2 = float(np.sum((ref - run) ** 2) / run.size)
    ref_max = float(np.max(ref))
    ref_sq = float(np.sum(ref ** 2))
    return {"mean_ref": float(np.mean(ref)), "mean_run": float(np.mean(run)), "e_inf": e_inf, "e_2": e_2,
            "relative_e_inf": e_inf / ref_max if ref_max != 0 else float("nan"),
            "relative_e_2": ref.size * e_2 / ref_sq if ref_sq != 0 else float("nan")}


def compare_fields(ref_path: str, run_path: str, component: str) -> Dict[str, Dict[str, float]]:
    """Read and compare the run's fields with the dataset's reference outputs
    (src/drivers/core.py:83-178); reference variables absent from the dataset
    are skipped with a log line."""
    ref_r, run_r = NetCDFReader(ref_path), NetCDFReader(run_path)
    keys = KEYS_ICE_ADJUST if component == "ice_adjust" else KEYS_RAIN_ICE
    metrics = {}
    for run_name, ref_name in keys:
        if ref_name not in ref_r or run_name not in run_r:
            log.info("field %s: %s not in both datasets, skipped", run_name, ref_name)
            continue
        run_field = run_r.get_field(run_name)
        ref_field = ref_r.get_field(ref_name)
        if run_name in TENDENCIES and ref_name == "PRS_OUT":
            # species stack, vapour first: rvs -> 0, rcs -> 1, ...
            ref_field = ref_field[:, TENDENCIES.index(run_name) - 1, :, :]
        if ref_field.shape != run_field.shape:
            log.info("field %s: shapes %s / %s differ, skipped", run_name, ref_field.shape, run_field.shape)
            continue
        metrics[run_name] = field_metrics(ref_field, run_field)
    ref_r.close()
    run_r.close()
    return metrics


def write_performance_tracking(exec_info: Dict, metrics: Dict, tracking_file: str) -> None:
    """{"performances": exec_info, "metrics": metrics} as JSON (src/drivers/core.py:41-66)."""
    def conv(o):
        if isinstance(o, dict):
            return {k: conv(v) for k, v in o.items()}
        if isinstance(o, (list, tuple)):
            return [conv(v) for v in o]
        if hasattr(o, "item"):
            return o.item()
        return o
    with open(tracking_file, "w") as fh:
        json.dump({"performances": conv(exec_info), "metrics": conv(metrics)}, fh, indent=2)


# ---------------------------------------------------------------------------- states

def ice_adjust_state_from_dataset(r: NetCDFReader) -> Dict[str, np.ndarray]:
    """IceAdjust arguments from a testprogs dataset (the mapping of
    tests/components/test_ice_adjust_jax.py:455-500), layout (ngpblks, nproma, nflevg)."""
    zrs = r.get_field("ZRS")                                   # (ngpblks, krr1, nproma, nflevg), theta first
    prs = r.get_field("PRS")                                   # (ngpblks, krr, nproma, nflevg), vapour first
    shape = zrs.shape[:1] + zrs.shape[2:]
    st = {"pabs": r.get_field("PPABSM"), "th": zrs[:, 0], "rv": zrs[:, 1], "rc": zrs[:, 2], "rr": zrs[:, 3],
          "ri": zrs[:, 4], "rs": zrs[:, 5], "rg": zrs[:, 6], "exn": r.get_field("PEXNREF"),
          "exn_ref": r.get_field("PEXNREF"), "rho_dry_ref": r.get_field("PRHODREF"), "rvs": prs[:, 0],
          "rcs": prs[:, 1], "ris": prs[:, 3], "ths": r.get_field("PTHS"), "cf_mf": r.get_field("PCF_MF"),
          "rc_mf": r.get_field("PRC_MF"), "ri_mf": r.get_field("PRI_MF"), "sigs": r.get_field("PSIGS")}
    sq = r.get_field("ZSIGQSAT")                               # (ngpblks, nproma)
    st["sigqsat"] = np.broadcast_to(sq[:, :, None], shape).copy()
    return {k: np.ascontiguousarray(v, dtype=np.float64) for k, v in st.items()}


def rain_ice_state_from_dataset(r: NetCDFReader) -> Dict[str, np.ndarray]:
    """RainIce state from a testprogs dataset (the mapping of
    tests/components/test_rain_ice_jax.py:45-100 and test_rain_ice_fortran.py:74-125)."""
    prt = r.get_field("PRT")
    prs = r.get_field("PRS")
    shape = prt.shape[:1] + prt.shape[2:]
    st = {"exn": r.get_field("PEXNREF"), "exnref": r.get_field("PEXNREF"), "rhodref": r.get_field("PRHODREF"),
          "pres": r.get_field("PPABSM"), "dzz": r.get_field("PDZZ"), "th_t": r.get_field("PTHT"),
          "ci_t": r.get_field("PCIT"), "ths": r.get_field("PTHS"), "sigs": r.get_field("PSIGS")}
    for i, s in enumerate(("v", "c", "r", "i", "s", "g")):
        st[f"r{s}_t"] = prt[:, i]
        st[f"r{s}s"] = prs[:, i]
    zero = np.zeros(shape)
    for opt in ("PCLDFR", "PHLC_HRC", "PHLC_HCF", "PHLI_HRI", "PHLI_HCF"):
        key = opt[1:].lower()
        st[key] = r.get_field(opt) if opt in r else zero.copy()
    st["sea"] = np.zeros(shape[:2])
    st["town"] = np.zeros(shape[:2])
    return {k: np.ascontiguousarray(v, dtype=np.float64) for k, v in st.items()}


def _synthetic(domain: Tuple[int, int, int], seed: int, dt: float, precip: bool) -> Dict[str, np.ndarray]:
    """make_state fields reshaped to (ngpblks, nproma, nflevg)."""
    from .state import make_state
    g, p, z = domain
    st = make_state(g * p, z, seed=seed, precip=precip, dt=dt)

    def lay(v):
        v = v.numpy()
        return np.ascontiguousarray(v.T.reshape(g, p, z)) if v.ndim == 2 else v.reshape(g, p)
    return {k: lay(v) for k, v in st.items()}


# ---------------------------------------------------------------------------- commands

def _to_device(st: Dict[str, np.ndarray]):
    import torch
    return {k: torch.as_tensor(v).cuda() for k, v in st.items()}


def run_ice_adjust(domain=(10000, 1, 50), dataset: Optional[str] = None, output_path: str = "ice_adjust_run.nc",
                   tracking_file: str = "ice_adjust_run.json", backend: str = "ice3gb", dt: float = 50.0,
                   seed: int = 0, table: str = "jax") -> Dict:
    """The ``ice-adjust`` command (src/drivers/cli.py:29-200)."""
    import torch
    from .components import IA_INOUT, IA_OUTPUTS, IceAdjust
    if dataset:
        r = NetCDFReader(dataset)
        st = ice_adjust_state_from_dataset(r)
        r.close()
    else:
        s = _synthetic(tuple(domain), seed, dt, precip=False)
        st = {k: s[k] for k in ("pabs", "th", "rv", "rc", "rr", "ri", "rs", "rg", "exn", "exn_ref", "rho_dry_ref",
                                "rvs", "rcs", "ris", "ths", "cf_mf", "rc_mf", "ri_mf", "sigs")}
        st["sigqsat"] = np.broadcast_to(s["sigqsat"][:, :, None], st["th"].shape).copy()
    ia = IceAdjust(table=table)
    names = ("sigqsat", "pabs", "sigs", "th", "exn", "exn_ref", "rho_dry_ref", "rv", "rc", "ri", "rr", "rs", "rg",
             "cf_mf", "rc_mf", "ri_mf", "rvs", "rcs", "ris", "ths")
    if backend == "ice3gb":
        x = _to_device({k: st[k] for k in names})
        ia(**x, timestep=dt)                                   # first call: library load, handle
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = ia(**x, timestep=dt)
        torch.cuda.synchronize()
        elapsed = time.perf_counter() - t0
        res = [v.cpu().numpy() for v in res]
    elif backend == "ice3gb-host":
        x = {k: st[k] for k in names}
        ia(**x, timestep=dt)
        t0 = time.perf_counter()
        res = ia(**x, timestep=dt)
        elapsed = time.perf_counter() - t0
    else:
        raise ValueError(f"unknown backend {backend!r} (ice3gb, ice3gb-host)")
    out = dict(st)
    out.update(dict(zip(IA_OUTPUTS + IA_INOUT, res)))
    log.info("Execution duration for IceAdjust : %s s", elapsed)
    write_dataset(out, output_path)
    metrics = compare_fields(dataset, output_path, "ice_adjust") if dataset else {}
    perf = {"execution_time": elapsed, "backend": backend, "domain": list(st["th"].shape),
            "grid_points_per_s": st["th"].size / elapsed}
    write_performance_tracking(perf, metrics, tracking_file)
    return {"performances": perf, "metrics": metrics}


def run_rain_ice(domain=(5000, 1, 15), dataset: Optional[str] = None, output_path: str = "rain_ice_run.nc",
                 tracking_file: str = "rain_ice_run.json", backend: str = "ice3gb", dt: float = 50.0, seed: int = 0,
                 table: str = "phyex") -> Dict:
    """The ``rain-ice`` command (src/drivers/cli.py:203-309)."""
    import torch
    from .components import RainIce
    if dataset:
        r = NetCDFReader(dataset)
        st = rain_ice_state_from_dataset(r)
        r.close()
    else:
        from .state import rain_ice_state
        s = _synthetic(tuple(domain), seed, dt, precip=True)
        st = rain_ice_state(s)
    ri = RainIce(table=table, layout="jax")
    if backend == "ice3gb":
        x = _to_device(st)
        ri(x, dt, with_fluxes=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        new, diag = ri(x, dt, with_fluxes=True)
        torch.cuda.synchronize()
        elapsed = time.perf_counter() - t0
        new = {k: (v.cpu().numpy() if isinstance(v, torch.Tensor) else v) for k, v in new.items()}
        diag = {k: v.cpu().numpy() for k, v in diag.items()}
    elif backend == "ice3gb-host":
        ri(st, dt, with_fluxes=True)
        t0 = time.perf_counter()
        new, diag = ri(st, dt, with_fluxes=True)
        elapsed = time.perf_counter() - t0
    else:
        raise ValueError(f"unknown backend {backend!r} (ice3gb, ice3gb-host)")
    out = {k: np.asarray(v) for k, v in new.items()}
    shape = st["th_t"].shape
    for k, v in diag.items():
        if k.startswith("fpr_"):
            continue
        out[k] = v.reshape(shape[:2]) if v.ndim == 1 else v
    if "fpr_c" in diag:
        # PFPR layout: species stack with vapour first (index 0 unused)
        out["fpr"] = np.stack([np.zeros(shape)] + [diag[f"fpr_{s}"] for s in "crisg"], axis=1)
    log.info("Execution duration for RainIce : %s s", elapsed)
    write_dataset(out, output_path)
    metrics = compare_fields(dataset, output_path, "rain_ice") if dataset else {}
    perf = {"execution_time": elapsed, "backend": backend, "domain": list(shape),
            "grid_points_per_s": int(np.prod(shape)) / elapsed}
    write_performance_tracking(perf, metrics, tracking_file)
    return {"performances": perf, "metrics": metrics}


def main(argv: Optional[List[str]] = None) -> int:
    logging.basicConfig(level=logging.INFO, stream=sys.stdout)
    ap = argparse.ArgumentParser(prog="python -m ice3gb.drivers")
    sub = ap.add_subparsers(dest="cmd", required=True)
    for name, dom, comp in (("ice-adjust", (10000, 1, 50), "ice_adjust"), ("rain-ice", (5000, 1, 15), "rain_ice")):
        p = sub.add_parser(name)
        p.add_argument("--domain", type=int, nargs=3, default=list(dom), metavar=("NGPBLKS", "NPROMA", "NFLEVG"))
        p.add_argument("--dataset", default=None, help="testprogs netCDF-3 dataset (default: synthetic state)")
        p.add_argument("--output-path", default=f"{comp}_run.nc")
        p.add_argument("--tracking-file", default=f"{comp}_run.json")
        p.add_argument("--backend", default="ice3gb", choices=("ice3gb", "ice3gb-host"))
        p.add_argument("--dt", type=float, default=50.0)
        p.add_argument("--seed", type=int, default=0)
    a = ap.parse_args(argv)
    kw = dict(domain=a.domain, dataset=a.dataset, output_path=a.output_path, tracking_file=a.tracking_file,
              backend=a.backend, dt=a.dt, seed=a.seed)
    res = run_ice_adjust(**kw) if a.cmd == "ice-adjust" else run_rain_ice(**kw)
    print(json.dumps(res["performances"]))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
