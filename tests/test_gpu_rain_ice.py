"""Statistical sedimentation, rain_ice and the chained physics step on the
GPU: parity with the reference JAX (sedimentation) and with the oracle
(Fortran-following rain_ice), options, properties at full size, and the
device-side pass-cap status (failure detection without a GPU fault)."""
import ctypes

import numpy as np
import pytest
import torch

from conftest import assert_parity, load_golden, rel_err, sensitivity
from helpers import TOL

pytestmark = pytest.mark.gpu
DT = 50.0


def _np_state(nij, nk=90, seed=0):
    from ice3gb.state import make_state
    return {k: v.numpy() for k, v in make_state(nij, nk, seed=seed, precip=True).items()}


def _abi_rain_ice_state(st):
    """make_state names -> the ABI field names used by oracle.rain_ice."""
    m = {"exn": "exn", "dzz": "dzz", "rhodref": "rho_dry_ref", "exnref": "exn_ref", "pabs": "pabs",
         "cldfr": "cldfr", "sigs": "sigs", "tht": "th", "rvt": "rv", "rct": "rc", "rrt": "rr", "rit": "ri",
         "rst": "rs", "rgt": "rg", "cit": "ci_t", "hlc_hrc": "hlc_hrc", "hlc_hcf": "hlc_hcf", "hli_hri": "hli_hri",
         "hli_hcf": "hli_hcf", "ths": "ths", "rvs": "rvs", "rcs": "rcs", "rrs": "rrs", "ris": "ris", "rss": "rss",
         "rgs": "rgs", "sea": "sea", "town": "town"}
    return {k: st[v] for k, v in m.items()}


# ---------------------------------------------------------------- sedimentation

def test_sedimentation_matches_reference_jax_golden():
    import oracle
    from ice3gb import Sedimentation
    g = load_golden("sed_jax")
    i = {k[3:]: v for k, v in g.items() if k.startswith("in_")}
    sed = Sedimentation(semantics="jax")
    _, spread = sensitivity(lambda x: oracle.sedimentation(sed.table, x, DT, fortran=False, with_fpr=True), i)
    T = lambda x: torch.as_tensor(np.ascontiguousarray(x)).cuda()
    out = sed(T(i["rhodref"]), T(i["dzz"]), T(i["pabs"]), T(i["tht"]), T(i["rcs"]), T(i["rrs"]), T(i["ris"]),
              T(i["rss"]), T(i["rgs"]), sea=T(i["sea"]), town=T(i["town"]), dt=DT)
    names = ("rcs", "rrs", "ris", "rss", "rgs", "fpr_c", "fpr_r", "fpr_i", "fpr_s", "fpr_g", "inprc", "inprr",
             "inpri", "inprs", "inprg")
    for n, o in zip(names, out):
        assert_parity(o.cpu().numpy(), g[f"out_{n}"], spread[n], n)


def test_sedimentation_fortran_matches_oracle_and_closes_budget():
    import oracle
    from ice3gb import Sedimentation
    st = _np_state(48 * 48, seed=4)
    i = {"rhodref": st["rho_dry_ref"], "dzz": st["dzz"], "pabs": st["pabs"], "tht": st["th"],
         "rcs": st["rcs"], "rrs": st["rrs"], "ris": st["ris"], "rss": st["rss"], "rgs": st["rgs"]}
    sed = Sedimentation(table="phyex", semantics="phyex")
    ref, spread = sensitivity(lambda x: oracle.sedimentation(sed.table, x, DT, fortran=True, with_fpr=True), i)
    T = lambda x: torch.as_tensor(np.ascontiguousarray(x)).cuda()
    out = sed(*(T(i[k]) for k in ("rhodref", "dzz", "pabs", "tht", "rcs", "rrs", "ris", "rss", "rgs")), dt=DT)
    names = ("rcs", "rrs", "ris", "rss", "rgs", "fpr_c", "fpr_r", "fpr_i", "fpr_s", "fpr_g", "inprc", "inprr",
             "inpri", "inprs", "inprg")
    res = {n: o.cpu().numpy() for n, o in zip(names, out)}
    # a source after sedimentation is S + (F_{k+1} - F_k)/(rho dz): its scale
    # is that of the terms summed (mode_ice4_sedimentation_stat.F90:203-207)
    rhodz = i["rhodref"] * i["dzz"]
    for n in names:
        scale = None
        if n in ("rcs", "rrs", "ris", "rss", "rgs"):
            f = ref["fpr_" + {"rcs": "c", "rrs": "r", "ris": "i", "rss": "s", "rgs": "g"}[n]]
            fa = np.concatenate([f[1:], np.zeros_like(f[:1])], axis=0)
            scale = np.abs(i[n]) + (np.abs(f) + np.abs(fa)) / rhodz
        assert_parity(res[n], ref[n], spread[n], n, scale=scale)
    # column mass budget: sum_k rho dz (S_after - S_before) = -rho_lw * inpr, per species
    for s, p in zip(("rcs", "rrs", "ris", "rss", "rgs"), ("inprc", "inprr", "inpri", "inprs", "inprg")):
        rhodz_ = i["rhodref"] * i["dzz"]
        col = (rhodz_ * (res[s] - i[s])).sum(0)
        scale = (rhodz_ * (np.abs(res[s]) + np.abs(i[s]))).sum(0) + 1000.0 * np.abs(res[p]) + 1e-300
        assert np.max(np.abs(col + 1000.0 * res[p]) / scale) < 1e-12, s


# ---------------------------------------------------------------- rain_ice

@pytest.fixture(scope="module")
def rain_ice():
    from ice3gb import RainIce
    return RainIce()


def _run_gpu(ri, st, **kw):
    from ice3gb.state import rain_ice_state
    state = {k: (torch.as_tensor(np.ascontiguousarray(v)).cuda()) for k, v in rain_ice_state(
        {k: torch.as_tensor(v) for k, v in st.items()}).items()}
    new, diag = ri(state, DT, **kw)
    torch.cuda.synchronize()
    return {k: (v.cpu().numpy() if isinstance(v, torch.Tensor) else v) for k, v in {**new, **diag}.items()}


def _oracle_ri(table, st, **kw):
    """Oracle rain_ice and its conditioning spread on the same inputs.

    The ICE4 time splitting decides sub-steps on rounding-size residuals (a
    depleted species whose residual exceeds XRTMIN gets one more MNH_TINY
    pass, mode_ice4_stepping.F90:302-311), so at some points the reference's
    own output moves by up to ~1e-8 relative under input changes of 1e-12:
    the envelope is sampled with 6 perturbed runs."""
    import oracle
    abi = _abi_rain_ice_state(st)
    bits = []

    def fn(x):
        out, b = oracle.rain_ice(table, x, DT, **kw)
        bits.append(b)
        return out
    ref, spread = sensitivity(fn, abi, rel=1e-12, trials=6)
    assert bits[0] == 0
    # operand scale of the sources: S_out = S_in + microphysics + (F_{k+1}-F_k)/(rho dz)
    fl, _ = oracle.rain_ice(table, abi, DT, with_fpr=True, **kw)
    rhodz = abi["rhodref"] * abi["dzz"]
    ref["_scale"] = {}
    for s_, f_ in (("rcs", "c"), ("rrs", "r"), ("ris", "i"), ("rss", "s"), ("rgs", "g")):
        f = fl["fpr_" + f_]
        fa = np.concatenate([f[1:], np.zeros_like(f[:1])], axis=0)
        ref["_scale"][s_] = np.abs(abi[s_]) + np.abs(ref[s_]) + (np.abs(f) + np.abs(fa)) / rhodz
    for s_ in ("ths", "rvs"):
        ref["_scale"][s_] = np.abs(abi[s_]) + np.abs(ref[s_])
    # the other outcomes of the depletion ties (a rounding residual against
    # XRTMIN deciding one more MNH_TINY pass)
    ref["_alts"] = oracle.rain_ice_depletion_alternatives(table, abi, DT, **kw)
    return ref, spread


def _compare(out, ref, spread, skip=()):
    pairs = {"ths": "ths", "rvs": "rvs", "rcs": "rcs", "rrs": "rrs", "ris": "ris", "rss": "rss", "rgs": "rgs",
             "ci_t": "cit", "evap3d": "evap3d", "rainfr": "rainfr", "inprc": "inprc", "inprr": "inprr",
             "inpri": "inpri", "inprs": "inprs", "inprg": "inprg"}
    for mine, theirs in pairs.items():
        if mine in skip:
            continue
        assert_parity(out[mine], ref[theirs], spread[theirs], mine, scale=ref["_scale"].get(theirs),
                      alts=[a[theirs] for a in ref["_alts"]])


@pytest.mark.parametrize("seed,nij", [(0, 32 * 32), (3, 64 * 64)])
def test_rain_ice_matches_oracle(rain_ice, seed, nij):
    st = _np_state(nij, seed=seed)
    ref, spread = _oracle_ri(rain_ice.table, st)
    out = _run_gpu(rain_ice, st)
    _compare(out, ref, spread)
    assert rain_ice.device_status() == 0


@pytest.mark.parametrize("opts", [dict(lsedim_after=True), dict(ldeposc=True), dict(lfeedbackt=False)])
def test_rain_ice_options_match_oracle(rain_ice, opts):
    import oracle
    st = _np_state(24 * 24, seed=11)
    kw = dict(lsedim_after=int(opts.get("lsedim_after", False)), ldeposc=int(opts.get("ldeposc", False)),
              lfeedbackt=int(opts.get("lfeedbackt", True)))
    ref, spread = _oracle_ri(rain_ice.table, st, **kw)
    out = _run_gpu(rain_ice, st, **opts)
    _compare(out, ref, spread)


def test_rain_ice_jax_sedimentation_and_phyex_table():
    import oracle
    from ice3gb import RainIce
    st = _np_state(24 * 24, seed=12)
    ri = RainIce(table="jax", sedimentation="jax")
    ref, spread = _oracle_ri(ri.table, st, sed_jax=1)
    _compare(_run_gpu(ri, st), ref, spread)


def test_rain_ice_host_entry_point_equals_device(rain_ice):
    from ice3gb.state import rain_ice_state
    st = _np_state(20 * 20, seed=13)
    dev = _run_gpu(rain_ice, st)
    host_state = {k: np.ascontiguousarray(v.numpy()) for k, v in rain_ice_state(
        {k: torch.as_tensor(v) for k, v in st.items()}).items()}
    new, diag = rain_ice(host_state, DT)
    for k in ("ths", "rvs", "rcs", "rrs", "ris", "rss", "rgs", "ci_t"):
        np.testing.assert_array_equal(new[k], dev[k], err_msg=k)
    for k in ("inprr", "inprs", "evap3d", "rainfr"):
        np.testing.assert_array_equal(diag[k], dev[k], err_msg=k)


def test_rain_ice_full_size_properties(rain_ice):
    """256x256x90 (5.9M points): sources of the condensates non-negative after
    the correction, column water budget closed by the surface precipitation,
    finite outputs, determinism."""
    from ice3gb.state import make_state, rain_ice_state
    st = rain_ice_state(make_state(256 * 256, 90, seed=2, precip=True, device="cuda"))
    new, diag = rain_ice(st, DT)
    new2, diag2 = rain_ice(st, DT)
    for k in ("rcs", "rrs", "ris", "rss", "rgs"):
        assert float(new[k].min()) >= 0.0, k
        assert torch.equal(new[k], new2[k])
    for k, v in {**new, **diag}.items():
        if isinstance(v, torch.Tensor):
            assert bool(torch.isfinite(v).all()), k
    dS = sum(new[k] - st[k] for k in ("rvs", "rcs", "rrs", "ris", "rss", "rgs"))
    col = (st["rhodref"] * st["dzz"] * dS).sum(0)
    pr = 1000.0 * sum(diag[k] for k in ("inprc", "inprr", "inpri", "inprs", "inprg"))
    assert float((col + pr).abs().max() / pr.abs().max()) < 1e-12
    assert rain_ice.device_status() == 0


def test_pass_cap_sets_device_status(rain_ice):
    """max_iterations=1 cannot finish the sub-stepping of most points: the
    kernel stops them, sets the status bit and returns normally; the host sees
    ICE3GB_ERR_DEVICE through ice3gb_status and the context stays usable."""
    st = _np_state(16 * 16, seed=1)
    _run_gpu(rain_ice, st, max_iterations=1)
    assert rain_ice.device_status() & 1
    # the context is still usable and the bit was cleared
    _run_gpu(rain_ice, st)
    assert rain_ice.device_status() == 0


# ---------------------------------------------------------------- chained step

def _step_state(st):
    return {"sigqsat": st["sigqsat"], "pabs": st["pabs"], "exn": st["exn"], "exnref": st["exn_ref"],
            "rhodref": st["rho_dry_ref"], "dzz": st["dzz"], "sigs": st["sigs"], "th": st["th"], "rv": st["rv"],
            "rc": st["rc"], "ri": st["ri"], "rr": st["rr"], "rs": st["rs"], "rg": st["rg"], "cf_mf": st["cf_mf"],
            "rc_mf": st["rc_mf"], "ri_mf": st["ri_mf"], "sea": st["sea"], "town": st["town"], "ths": st["ths"],
            "rvs": st["rvs"], "rcs": st["rcs"], "rrs": st["rrs"], "ris": st["ris"], "rss": st["rss"],
            "rgs": st["rgs"], "cit": st["ci_t"]}


def _gpu_step(handle, st, host=False):
    from ice3gb import _abi
    nk, nij = st["pabs"].shape
    keep, f = {}, _abi.StepFields()
    conv = (lambda a: np.ascontiguousarray(a)) if host else (lambda a: torch.as_tensor(np.ascontiguousarray(a)).cuda())
    ptr = (lambda a: a.ctypes.data_as(ctypes.c_void_p)) if host else (lambda a: ctypes.c_void_p(a.data_ptr()))
    for k in _abi.STEP_IN + ("sea", "town") + _abi.STEP_INOUT:
        keep[k] = conv(st[k]).copy() if host else conv(st[k]).clone()
        setattr(f, k, ptr(keep[k]))
    for k in _abi.STEP_OUT3:
        keep[k] = np.empty((nk, nij)) if host else torch.empty((nk, nij), dtype=torch.float64, device="cuda")
        setattr(f, k, ptr(keep[k]))
    for k in _abi.STEP_OUT2:
        keep[k] = np.empty(nij) if host else torch.empty(nij, dtype=torch.float64, device="cuda")
        setattr(f, k, ptr(keep[k]))
    opt = _abi.RainIceOptions(-1, -1, -1, 0, 0)
    fn = handle.lib.ice3gb_physics_step_host if host else handle.lib.ice3gb_physics_step
    _abi.check(fn(handle.h, nij, nk, DT, ctypes.byref(opt), ctypes.byref(f),
                  ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), handle.h, "physics_step")
    torch.cuda.synchronize()
    return {k: (v if host else v.cpu().numpy()) for k, v in keep.items()}


def test_physics_step_matches_oracle_and_host_path():
    import oracle
    from ice3gb.components import Ice3Handle
    from ice3gb.constants import build_table
    table = build_table(table="phyex")
    h = Ice3Handle(table)
    st = _step_state(_np_state(32 * 32, seed=21))
    ref, spread = sensitivity(lambda x: oracle.physics_step(table, x, DT)[0], st, rel=1e-12, trials=6)
    out = _gpu_step(h, st)
    for k in ref:
        assert_parity(out[k], ref[k], spread[k], k)
    host = _gpu_step(h, st, host=True)
    for k in ref:
        np.testing.assert_array_equal(host[k], out[k], err_msg=k)



@pytest.mark.parametrize("nij", [128 * 128, 3 * 4096 + 100, 6 * 4096 + 64])
def test_physics_step_host_slab_pipeline_matches_device(nij):
    """The host entry point runs the step in column slabs (4096 columns and
    more, the first and last three graded down to a quarter when the grid
    holds six) on a copy-in, two compute and a copy-out stream; its outputs,
    evap3d's fix-up on the maximum
    pass key of the whole call included, equal the device entry point's bit
    for bit, also with a ragged slab."""
    from ice3gb.components import Ice3Handle
    from ice3gb.constants import build_table
    h = Ice3Handle(build_table(table="phyex"))
    st = _step_state(_np_state(nij, seed=4))
    dev = _gpu_step(h, st)
    host = _gpu_step(h, st, host=True)
    for k in dev:
        np.testing.assert_array_equal(host[k], dev[k], err_msg=k)
    assert h.status() == 0


@pytest.mark.parametrize("accr,evap,aucv_rc,aucv_ri", [(1, 2, 3, 1), (0, 1, 1, 0), (1, 0, 3, 0), (0, 2, 3, 1)])
def test_rain_ice_subgrid_warm_options_match_oracle(accr, evap, aucv_rc, aucv_ri):
    """SUBG_RC_RR_ACCR / SUBG_RR_EVAP other than NONE on the device: the
    precipitation-fraction column kernel, then the point kernel's subgrid
    instantiation, against the oracle's RAIN_ICE (sources, ci_t, evap3d,
    the precipitation fraction and the partitions the PRFR set-up rewrites)."""
    from ice3gb import RainIce
    from ice3gb.constants import build_table
    ri = RainIce()
    ri.table = build_table(table="phyex", overrides={"SUBG_RC_RR_ACCR": accr, "SUBG_RR_EVAP": evap,
                                                     "SUBG_AUCV_RC": aucv_rc, "SUBG_AUCV_RI": aucv_ri})
    st = _np_state(32 * 32, seed=21)
    ref, spread = _oracle_ri(ri.table, st)
    out = _run_gpu(ri, st)
    _compare(out, ref, spread)
    for k in ("hlc_hcf", "hlc_hrc", "hli_hcf", "hli_hri"):
        assert_parity(out[k], ref[k], spread[k], k)
    assert ri.device_status() == 0


@pytest.mark.parametrize("lsedim_after", [False, True])
def test_rain_ice_split_sedimentation_matches_oracle(lsedim_after):
    """SEDIM = SPLI: the time-split sedimentation column kernel (with its
    negativity correction) inside rain_ice, before or after the
    microphysics, against the oracle's RAIN_ICE."""
    from ice3gb import RainIce
    from ice3gb.constants import build_table
    ri = RainIce()
    ri.table = build_table(table="phyex", overrides={"SEDIM": 0.0})
    st = _np_state(32 * 32, seed=23)
    ref, spread = _oracle_ri(ri.table, st, lsedim_after=int(lsedim_after))
    out = _run_gpu(ri, st, lsedim_after=lsedim_after)
    _compare(out, ref, spread)
    assert ri.device_status() == 0
    assert np.count_nonzero(out["inprr"]) > 100

