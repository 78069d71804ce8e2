#!/usr/bin/env python
"""Benchmark of the ICE3 hot path on GB300.

Workload (default "chain"): one chained microphysics step
    S1 = ice_adjust(x_t, S0); S2 = rain_ice(x_t, S1); S3 = ice_adjust(dt S2, S2)
(PHYEX total sources: dt*S2 is the state after the microphysics)
on 1024 x 1024 columns x 90 levels (94,371,840 grid points), FP64, dt = 50 s,
seeded synthetic AROME-like state, through ice3gb_physics_step.

Metric: grid-points/s (points of the step / step time).
  value : inputs resident in HBM, device time of K steps (CUDA events on the
          launching stream, W warm-up steps before).  Each step first restores
          the 8 in-out fields (7 sources + ci_t) from pristine device copies so
          every step does identical work; those copies are inside the timed
          region.  Inputs are far larger than L2 (no flush needed).
  e2e   : the same step through the host-buffer C-ABI entry point
          ice3gb_physics_step_host with pinned host buffers (h2d of the inputs,
          the kernels, d2h of the results, per step).
  roofline: dominant kernel's algorithmic bytes per launch / its average
          launch time (CUDA events around each launch on the launching stream),
          against the measured HBM copy bandwidth.
  cpu_baseline: the CPU oracle (C, OpenMP, all host cores) on the same whole
          state, one warm-up then at least 2 steps (about 10 s).
  --impl reference: the same oracle (the reference's own code cannot run on
          the box) on the same workload, W warm-up and K timed steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "dwarf-p-ice3_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

DT = 50.0
NK = 90
METRIC = "grid-points/s ice_adjust+rain_ice (chained ice_adjust->rain_ice->ice_adjust step)"

# Algorithmic bytes per grid point (each distinct field read or written once, 8 B):
#  chained step: 24 3-D fields read, 19 written -> 344 B
#  ice_adjust  : 19 read (+ sigqsat per column), 16 written -> 280 B
#  rain_ice pointwise kernel: 20 read (exn exnref rhodref pabs cldfr sigs th rv rc rr ri rs rg cit,
#      7 sources minus one counted once) / 10 written (7 sources, cit, evap3d, rainfr) -> 240 B
#  sedimentation: 9 read (rhodref dzz pabs th + 5 sources), 5 written -> 112 B
ALGO_BYTES = {"chain": 344, "ice_adjust": 280, "rain_ice": 240, "sedimentation": 112,
              "rain_ice_evap_fixup": 4, "fog_deposition": 0}
STEP_IN = ("sigqsat", "pabs", "exn", "exnref", "rhodref", "dzz", "sigs", "th", "rv", "rc", "ri", "rr", "rs", "rg",
           "cf_mf", "rc_mf", "ri_mf")
STEP_INOUT = ("ths", "rvs", "rcs", "rrs", "ris", "rss", "rgs", "cit")
STEP_OUT3 = ("t", "rv_out", "rc_out", "ri_out", "cldfr", "hlc_hrc", "hlc_hcf", "hli_hri", "hli_hcf", "evap3d",
             "rainfr")
STEP_OUT2 = ("inprc", "inprr", "inpri", "inprs", "inprg")


def step_state(st):
    """make_state(..., precip=True) names -> StepFields names."""
    m = {"sigqsat": "sigqsat", "pabs": "pabs", "exn": "exn", "exnref": "exn_ref", "rhodref": "rho_dry_ref",
         "dzz": "dzz", "sigs": "sigs", "th": "th", "rv": "rv", "rc": "rc", "ri": "ri", "rr": "rr", "rs": "rs",
         "rg": "rg", "cf_mf": "cf_mf", "rc_mf": "rc_mf", "ri_mf": "ri_mf", "sea": "sea", "town": "town",
         "ths": "ths", "rvs": "rvs", "rcs": "rcs", "rrs": "rrs", "ris": "ris", "rss": "rss", "rgs": "rgs",
         "cit": "ci_t"}
    return {k: st[v] for k, v in m.items()}


def load_peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        self.fh.close()

    def summary(self):
        rows = []
        try:
            with open(self.path) as fh:
                for line in fh:
                    parts = [x.strip() for x in line.split(",")]
                    if len(parts) >= 9:
                        rows.append(parts)
            os.unlink(self.path)
        except Exception:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max((float(r[3]) for r in rows if r[3].replace(".", "").isdigit()), default=None)}


# ----------------------------------------------------------------------------- CPU side

def workload_config(nij, seed):
    """The workload named in both arms' JSON lines (the same for each)."""
    n = nij * NK
    return {"workload": f"chained ice_adjust->rain_ice->ice_adjust, {nij} columns x {NK} levels "
                        f"({n} grid points) per GPU, FP64, dt={DT}s, AROME table (PHYEX values)",
            "columns_per_gpu": nij, "levels": NK, "dt": DT, "seed": seed,
            "l2": "inputs larger than L2 (no flush)"}


def cpu_chain_steps(st_np, steps, warmup=1, budget_s=None):
    """The oracle's chained step on the host cores (C, OpenMP, all threads) on
    the whole state `st_np`: `warmup` untimed steps, then `steps` timed ones
    (or, with `budget_s`, at least `steps` and until the budget is spent).
    Outputs are allocated once; each step starts from the same in-out fields;
    the time is the step call alone.  Returns the per-step times."""
    import oracle
    from ice3gb.constants import build_table

    table = build_table(table="phyex")
    out = None
    for _ in range(max(warmup, 1)):
        out, _ = oracle.physics_step(table, st_np, DT, out=out)
    times = []
    t_start = time.perf_counter()
    while len(times) < steps or (budget_s is not None and time.perf_counter() - t_start < budget_s
                                 and len(times) < 50):
        oracle.physics_step(table, st_np, DT, out=out, elapsed=times)
    return times


def host_state(nij, seed):
    """The benchmark's state in host memory: generated on the GPU like the GPU
    arm's (the same numbers) when one is visible, else on the host (the same
    distributions, other draws)."""
    import torch

    from ice3gb.state import make_state
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    st = step_state(make_state(nij, NK, seed=seed, precip=True, device=dev))
    out = {k: v.cpu().numpy() for k, v in st.items()}
    del st
    if dev == "cuda":
        torch.cuda.empty_cache()
    return out, dev


def run_reference(args):
    """--impl reference: the reference path's CPU restatement (the oracle port;
    the reference's own Fortran and JAX code cannot run on the box) on the
    whole workload, every host core, `warmup` untimed then `steps` timed
    steps."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    st, dev = host_state(args.nij, args.seed)
    times = cpu_chain_steps(st, args.steps, warmup=args.warmup)
    pts = args.nij * NK
    total = sum(times)
    value = pts * len(times) / total
    cores = os.cpu_count()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "grid-points/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded AROME-like states)", "config": workload_config(args.nij, args.seed),
        "cpu_baseline": {"value": value, "unit": "grid-points/s", "cores": cores, "kind": "port",
                         "sample": f"the whole workload, {pts} points per step (state generated on the {dev}), "
                                   f"C/OpenMP over {cores} threads; the reference's PHYEX Fortran and JAX code "
                                   f"cannot run on the box"},
        "e2e": {"value": value, "unit": "grid-points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------------------- GPU side

def run_ours(args):
    import numpy as np
    import torch

    from ice3gb import _abi
    from ice3gb.components import Ice3Handle
    from ice3gb.constants import build_table
    from ice3gb.state import make_state

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    nij = args.nij
    n = nij * NK
    dev = torch.device("cuda", local)
    st = step_state(make_state(nij, NK, seed=args.seed + rank, precip=True, device=dev))
    pristine = {k: st[k].clone() for k in STEP_INOUT}
    work = {k: st[k].clone() for k in STEP_INOUT}
    outs = {k: torch.empty((NK, nij), dtype=torch.float64, device=dev) for k in STEP_OUT3}
    outs.update({k: torch.empty((nij,), dtype=torch.float64, device=dev) for k in STEP_OUT2})
    table = build_table(table="phyex")
    handle = Ice3Handle(table)
    lib = handle.lib
    f = _abi.StepFields()
    for k in STEP_IN + ("sea", "town"):
        setattr(f, k, ctypes.c_void_p(st[k].data_ptr()))
    for k, v in {**work, **outs}.items():
        setattr(f, k, ctypes.c_void_p(v.data_ptr()))
    opt = _abi.RainIceOptions(-1, -1, -1, 0, 0)
    stream = torch.cuda.current_stream(dev)
    sptr = ctypes.c_void_p(stream.cuda_stream)

    def step():
        for k in STEP_INOUT:
            work[k].copy_(pristine[k], non_blocking=True)
        _abi.check(lib.ice3gb_physics_step(handle.h, nij, NK, DT, ctypes.byref(opt), ctypes.byref(f), sptr),
                   handle.h, "ice3gb_physics_step")

    for _ in range(args.warmup):
        step()
    bits = handle.status()
    barrier()
    lib.ice3gb_profile_enable(handle.h, 1)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        barrier()
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        barrier()
    ms_total = ev0.elapsed_time(ev1)
    kstats = {}
    launches_total = 0
    for kid, name in enumerate(_abi.KERNEL_NAMES):
        cnt, tot = ctypes.c_int(0), ctypes.c_double(0.0)
        _abi.check(lib.ice3gb_profile_read(handle.h, kid, ctypes.byref(cnt), ctypes.byref(tot)), handle.h, "profile")
        if cnt.value:
            kstats[name] = {"launches": cnt.value, "total_ms": tot.value, "avg_ms": tot.value / cnt.value}
            launches_total += cnt.value
    lib.ice3gb_profile_enable(handle.h, 0)
    bits |= handle.status()
    if dist is not None:
        t = torch.tensor([ms_total], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_total = float(t.item())
    ms_step = ms_total / args.steps
    value = world * n / (ms_step / 1e3)

    # roofline of the dominant kernel
    peak, peak_kind = load_peaks()
    dom = max(kstats.items(), key=lambda kv: kv[1]["total_ms"])
    dom_name, dom_st = dom
    bytes_launch = ALGO_BYTES[dom_name] * n
    achieved = bytes_launch / (dom_st["avg_ms"] / 1e3) / 1e9
    traffic, fp64_pct = None, None
    tpath = os.path.join(REPO, "profiles", "traffic_per_point.txt")
    if os.path.exists(tpath):
        # "<kernel> <DRAM bytes per point>" and "fp64_pipe_pct <kernel> <pct>" lines
        # summarised from an ncu capture of the same kernels
        for line in open(tpath):
            w = line.split()
            if len(w) == 2 and w[0] == dom_name:
                traffic = float(w[1]) * n
            elif len(w) == 3 and w[0] == "fp64_pipe_pct" and w[1] == dom_name:
                fp64_pct = float(w[2])
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "kernel": dom_name, "peak_source": f"hbm_gbs of {peak_kind}",
                "algorithmic_bytes_per_launch": bytes_launch,
                # the bound that binds: GB300 FP64 issue rate (ncu pipe utilisation of this kernel)
                "fp64_pipe_pct_ncu": fp64_pct,
                "kernels": kstats}

    # surrogate-assisted step (the metric's second arm), then e2e through the
    # host-buffer entry point
    surrogate = None
    if not args.no_surrogate:
        surrogate = run_surrogate(args, lib, handle, st, f, work, pristine, outs, opt, nij, n, dev, stream, world,
                                  dist, value)
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, lib, handle, st, opt, nij, n, dev, world, dist)

    line = {
        "metric": METRIC, "value": value, "unit": "grid-points/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded AROME-like states)",
        "config": workload_config(nij, args.seed),
        "timed_step": "restore 8 in-out fields (device copies) + ice3gb_physics_step",
        "gpu_launches": launches_total, "device_status_bits": bits,
        "roofline": roofline, "clocks": clocks.summary(), "e2e": e2e, "surrogate": surrogate,
    }
    if not args.no_cpu and rank == 0:
        # the oracle's chained step on the same (whole) state, host cores
        st_cpu = {k: v.cpu().numpy() for k, v in st.items()}
        for k in STEP_INOUT:
            st_cpu[k] = pristine[k].cpu().numpy()
        ctimes = cpu_chain_steps(st_cpu, 2, warmup=1, budget_s=args.cpu_seconds)
        del st_cpu
        cval = n / statistics.median(ctimes)
        line["cpu_baseline"] = {"value": cval, "unit": "grid-points/s", "cores": os.cpu_count(), "kind": "port",
                                "sample": f"the whole workload ({n} points), {len(ctimes)} steps after one "
                                          f"warm-up, median step {statistics.median(ctimes):.3f}s"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


# forward FLOPs per point of the surrogate network 16 -> 256 x 3 -> 10
MLP_FLOP_PER_ROW = 2 * (16 * 256 + 2 * 256 * 256 + 256 * 10)
SUR_FIELDS = ("ths", "rvs", "rcs", "rrs", "ris", "rss", "rgs", "t", "rv_out", "rc_out", "ri_out", "cldfr")


def run_surrogate(args, lib, handle, st, f, work, pristine, outs, opt, nij, n, dev, stream, world, dist,
                  plain_value):
    """The chained step with the learned ICE4_SLOW rates
    (ice3gb_physics_step_surrogate) on the same state: device time per step,
    counters, the error per field against the plain FP64 step, per-tendency
    RMSE of the network against the plain kernel's rates on a column sample,
    and the tensor-core roofline of the network kernel."""
    import torch

    from ice3gb import _abi
    from ice3gb.surrogate import DEFAULT_PATH, SlowSurrogate, physics_step_surrogate

    if not os.path.exists(DEFAULT_PATH):
        return {"unavailable": "no trained surrogate in the package"}
    sur = SlowSurrogate.load(DEFAULT_PATH)

    def restore():
        for k in STEP_INOUT:
            work[k].copy_(pristine[k], non_blocking=True)

    def fields():
        return {**work, **outs}

    # one plain step and one surrogate step on identical inputs
    restore()
    _abi.check(lib.ice3gb_physics_step(handle.h, nij, NK, DT, ctypes.byref(opt), ctypes.byref(f),
                                       ctypes.c_void_p(stream.cuda_stream)), handle.h, "ice3gb_physics_step")
    plain = {k: fields()[k].clone() for k in SUR_FIELDS}
    restore()
    stats = physics_step_surrogate(handle, sur, f, nij, NK, DT, opt)
    err = {}
    for k in SUR_FIELDS:
        ref = plain[k]
        d = (fields()[k] - ref).double()
        base = pristine[k] if k in pristine else None
        scale = torch.sqrt(((ref - base) ** 2).mean()) if base is not None else torch.sqrt((ref ** 2).mean())
        err[k] = {"rmse": float(torch.sqrt((d * d).mean())), "nrmse": float(torch.sqrt((d * d).mean()) / scale),
                  "max_abs": float(d.abs().max())}
    del plain
    # timing (each call synchronises the stream twice: batch sizing, counters)
    for _ in range(2):
        restore()
        physics_step_surrogate(handle, sur, f, nij, NK, DT, opt)
    ksteps = max(2, min(args.steps, 4))
    lib.ice3gb_profile_enable(handle.h, 1)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(ksteps):
        restore()
        physics_step_surrogate(handle, sur, f, nij, NK, DT, opt)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / ksteps
    if dist is not None:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    kst = {}
    for kid, name in enumerate(_abi.KERNEL_NAMES):
        cnt, tot = ctypes.c_int(0), ctypes.c_double(0.0)
        _abi.check(lib.ice3gb_profile_read(handle.h, kid, ctypes.byref(cnt), ctypes.byref(tot)), handle.h, "profile")
        if cnt.value:
            kst[name] = {"launches": cnt.value, "total_ms": tot.value, "avg_ms": tot.value / cnt.value}
    lib.ice3gb_profile_enable(handle.h, 0)
    rows = stats["used"] + stats["fixup_fallback"]
    mlp = kst.get("surrogate_mlp")
    bf16_peak = None
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as fh:
            bf16_peak, peak_kind = float(json.load(fh)["bf16_tflops"]), "measured"
    except Exception:
        bf16_peak, peak_kind = 1900.0, "fallback"
    mlp_roof = None
    if mlp:
        ach = rows * MLP_FLOP_PER_ROW / (mlp["avg_ms"] / 1e3) / 1e12
        mlp_roof = {"bound": "tensor", "achieved": ach, "peak": bf16_peak, "unit": "TFLOP/s", "frac": ach / bf16_peak,
                    "peak_source": f"bf16_tflops of {peak_kind}", "rows_per_launch": rows,
                    "flop_per_row": MLP_FLOP_PER_ROW}
    # per-tendency error of the network on a column sample (plain kernel's rates as truth)
    tend = None
    try:
        from ice3gb.state import make_state
        from ice3gb.surrogate import training_set
        raw, tgt = training_set(1 << 20, nij=16384, seed=700000 + args.seed)
        tend = sur.rate_errors(raw, tgt)
    except Exception as e:  # noqa: BLE001
        tend = {"error": repr(e)}
    value = world * n / (ms / 1e3)
    return {"metric": METRIC + ", surrogate-assisted (learned ICE4_SLOW rates)", "value": value,
            "unit": "grid-points/s", "ms_per_step": ms, "steps": ksteps, "vs_plain": value / plain_value,
            "counters": stats, "field_error_vs_plain_fp64": err, "tendency_error_vs_plain": tend,
            "kernels": kst, "mlp_roofline": mlp_roof,
            "network": "16 -> 256 x 3 (GELU) -> 10, BF16 weights/activations, FP32 accumulation (tcgen05), "
                       "trained on 2^24 plain-kernel points",
            "timed_step": "restore 8 in-out fields + ice3gb_physics_step_surrogate (features, network, "
                          "rain_ice with learned slow rates and in-launch fallback, ice_adjust x2, sedimentation)"}


def run_e2e(args, lib, handle, st, opt, nij, n, dev, world, dist):
    import torch

    from ice3gb import _abi

    host = {k: v.cpu().pin_memory() for k, v in st.items()}
    pristine = {k: host[k].clone() for k in STEP_INOUT}
    outs = {k: torch.empty((NK, nij), dtype=torch.float64).pin_memory() for k in STEP_OUT3}
    outs.update({k: torch.empty((nij,), dtype=torch.float64).pin_memory() for k in STEP_OUT2})
    f = _abi.StepFields()
    for k, v in {**host, **outs}.items():
        setattr(f, k, ctypes.c_void_p(v.data_ptr()))
    stream = torch.cuda.current_stream(dev)
    sptr = ctypes.c_void_p(stream.cuda_stream)
    h2d = 8 * (sum(host[k].numel() for k in STEP_IN + ("sea", "town") + STEP_INOUT))
    d2h = 8 * (sum(host[k].numel() for k in STEP_INOUT) + sum(v.numel() for v in outs.values()))

    def call():
        _abi.check(lib.ice3gb_physics_step_host(handle.h, nij, NK, DT, ctypes.byref(opt), ctypes.byref(f), sptr),
                   handle.h, "ice3gb_physics_step_host")

    for _ in range(max(1, min(args.warmup, 2))):
        for k in STEP_INOUT:
            host[k].copy_(pristine[k])
        call()
    total = 0.0
    per_step = []
    for _ in range(args.steps):
        for k in STEP_INOUT:
            host[k].copy_(pristine[k])                    # restore in-out host fields (untimed)
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        call()                                            # h2d + kernels + d2h, synchronous
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        if dist is not None:
            t = torch.tensor([ms], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        total += ms
        per_step.append(ms)
    ms_step = total / args.steps
    del host, pristine, outs
    bw = copy_bandwidth(dev)
    return {"value": world * n / (ms_step / 1e3), "unit": "grid-points/s", "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h, "ms_per_step": ms_step,
            "step_ms_min_max": [min(per_step), max(per_step)],
            "step_ms": [round(x, 1) for x in per_step],
            "path": "ice3gb_physics_step_host, pinned host buffers",
            # the box's pinned-copy bandwidth, measured right after: the copies alone, one
            # direction after the other, would take h2d / h2d_gbs + d2h / d2h_gbs
            "copy_gbs": bw, "copies_alone_ms": 1e3 * (h2d / (bw["h2d"] * 1e9) + d2h / (bw["d2h"] * 1e9))}


def copy_bandwidth(dev, nbytes=1 << 30, reps=3):
    """Best-of-reps GB/s of one pinned host <-> device copy of nbytes each way."""
    import torch

    h = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    d = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    out = {}
    for name, dst, src in (("h2d", d, h), ("d2h", h, d)):
        best = None
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            dst.copy_(src, non_blocking=True)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        out[name] = nbytes / (best * 1e-3) / 1e9
    del h, d
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--nij", type=int, default=1024 * 1024)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-surrogate", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)   # timing rule: at least 3 warm-up steps
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.gpus != world:
        # one process per GPU: N > 1 comes from torchrun (WORLD_SIZE = N)
        print(f"bench.py: --gpus {args.gpus} needs {args.gpus} ranks (torchrun --nproc-per-node {args.gpus}); "
              f"WORLD_SIZE is {world}", file=sys.stderr)
        return 2
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
