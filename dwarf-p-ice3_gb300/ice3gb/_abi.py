"""ctypes binding of the C ABI declared in include/ice3gb.h.

The shared library ``libice3gb.so`` is built in-tree by
``dwarf-p-ice3_gb300/build.py`` (nvcc, sm_103a).  Loading fails loudly when it
is missing: there is no CPU fallback for the product path.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

from .constants import CONSTANT_NAMES, Ice3gbConstants, Ice3gbLuts  # noqa: F401

_HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.normpath(os.path.join(_HERE, ".."))
LIB_PATH = os.path.join(PKG_ROOT, "lib", "libice3gb.so")

P = ctypes.c_void_p

ICE3GB_OK = 0
ERRORS = {
    -1: "ICE3GB_ERR_NULL", -2: "ICE3GB_ERR_SHAPE", -3: "ICE3GB_ERR_ALIGN", -4: "ICE3GB_ERR_CUDA",
    -5: "ICE3GB_ERR_UNSUPPORTED", -6: "ICE3GB_ERR_DEVICE", -7: "ICE3GB_ERR_HANDLE", -8: "ICE3GB_ERR_RANGE",
}
DEV_PASS_CAP = 1


class IceAdjustFields(ctypes.Structure):
    _fields_ = [(n, P) for n in (
        "sigqsat", "pabs", "sigs", "th", "exn", "exn_ref", "rho_dry_ref",
        "rv", "rc", "ri", "rr", "rs", "rg", "cf_mf", "rc_mf", "ri_mf",
        "rvs", "rcs", "ris", "ths",
        "t", "rv_out", "rc_out", "ri_out", "cldfr",
        "hlc_hrc", "hlc_hcf", "hli_hri", "hli_hcf", "cph", "lv", "ls")] + [("sigqsat_3d", ctypes.c_int64),
                                                                         ("srcs", P)] + [
        (n, P) for n in ("zz", "ice_cld_wgt", "icldfr", "wcldfr", "ssio", "ssiu", "ifr")]

# outputs of the OCND2 option of ice_adjust, in the order of IceAdjustFields
OCND2_OUTPUTS = ("icldfr", "wcldfr", "ssio", "ssiu", "ifr")


class SedimentationFields(ctypes.Structure):
    _fields_ = [(n, P) for n in (
        "rhodref", "dzz", "pabs", "tht", "sea", "town",
        "rcs", "rrs", "ris", "rss", "rgs",
        "inprc", "inprr", "inpri", "inprs", "inprg",
        "fpr_c", "fpr_r", "fpr_i", "fpr_s", "fpr_g")] + [("fortran_semantics", ctypes.c_int64)]


class RainIceFields(ctypes.Structure):
    _fields_ = [(n, P) for n in (
        "exn", "dzz", "rhodref", "exnref", "pabs", "cldfr", "sigs",
        "tht", "rvt", "rct", "rrt", "rit", "rst", "rgt", "sea", "town",
        "cit", "hlc_hrc", "hlc_hcf", "hli_hri", "hli_hcf",
        "ths", "rvs", "rcs", "rrs", "ris", "rss", "rgs",
        "evap3d", "rainfr", "inprc", "inprr", "inpri", "inprs", "inprg", "indep",
        "fpr_c", "fpr_r", "fpr_i", "fpr_s", "fpr_g",
        "rht", "rhs", "inprh", "fpr_h",           # hail, NRR = 7
        "ssio", "ssiu", "ifr", "icldfr")]         # OCND2


class StepFields(ctypes.Structure):
    _fields_ = [(n, P) for n in (
        "sigqsat", "pabs", "exn", "exnref", "rhodref", "dzz", "sigs",
        "th", "rv", "rc", "ri", "rr", "rs", "rg", "cf_mf", "rc_mf", "ri_mf", "sea", "town",
        "ths", "rvs", "rcs", "rrs", "ris", "rss", "rgs", "cit",
        "t", "rv_out", "rc_out", "ri_out", "cldfr", "hlc_hrc", "hlc_hcf", "hli_hri", "hli_hcf",
        "evap3d", "rainfr", "inprc", "inprr", "inpri", "inprs", "inprg")]


IA_IN = ("sigqsat", "pabs", "sigs", "th", "exn", "exn_ref", "rho_dry_ref", "rv", "rc", "ri", "rr", "rs", "rg",
         "cf_mf", "rc_mf", "ri_mf", "rvs", "rcs", "ris", "ths")
IA_OUT = ("t", "rv_out", "rc_out", "ri_out", "cldfr", "hlc_hrc", "hlc_hcf", "hli_hri", "hli_hcf", "cph", "lv", "ls",
          "rvs", "rcs", "ris", "ths")


class SedimentationCotangents(ctypes.Structure):
    _fields_ = [(n, P) for n in ("rcs", "rrs", "ris", "rss", "rgs", "inprc", "inprr", "inpri", "inprs", "inprg",
                                 "fpr_c", "fpr_r", "fpr_i", "fpr_s", "fpr_g")]


class SedimentationGradients(ctypes.Structure):
    _fields_ = [(n, P) for n in ("rcs", "rrs", "ris", "rss", "rgs", "rhodref", "dzz", "pabs", "tht")]


class IceAdjustCotangents(ctypes.Structure):
    _fields_ = [(n, P) for n in IA_OUT]


class IceAdjustGradients(ctypes.Structure):
    _fields_ = [(n, P) for n in IA_IN]


STEP_IN = ("sigqsat", "pabs", "exn", "exnref", "rhodref", "dzz", "sigs", "th", "rv", "rc", "ri", "rr", "rs", "rg",
           "cf_mf", "rc_mf", "ri_mf")
STEP_INOUT = ("ths", "rvs", "rcs", "rrs", "ris", "rss", "rgs", "cit")
STEP_OUT3 = ("t", "rv_out", "rc_out", "ri_out", "cldfr", "hlc_hrc", "hlc_hcf", "hli_hri", "hli_hcf", "evap3d",
             "rainfr")
STEP_OUT2 = ("inprc", "inprr", "inpri", "inprs", "inprg")


class MlpShape(ctypes.Structure):
    _fields_ = [("n_in", ctypes.c_int32), ("n_hidden", ctypes.c_int32),
                ("n_hidden_layers", ctypes.c_int32), ("n_out", ctypes.c_int32)]


class SurrogateNorm(ctypes.Structure):
    _fields_ = [("mean", ctypes.c_float * 16), ("inv_std", ctypes.c_float * 16), ("lo", ctypes.c_float * 16),
                ("hi", ctypes.c_float * 16)]


# counters of the surrogate calls (ICE3GB_SUR_*)
SUR_STATS = ("micro", "outside_envelope", "over_capacity", "used", "fixup_fallback")
SUR_NSTATS = 8


class RainIceOptions(ctypes.Structure):
    _fields_ = [("lsedim_after", ctypes.c_int32), ("ldeposc", ctypes.c_int32),
                ("lfeedbackt", ctypes.c_int32), ("max_passes", ctypes.c_int32),
                ("sed_jax", ctypes.c_int32)]


EXPORTED = (
    "ice3gb_version", "ice3gb_constant_count", "ice3gb_constant_name", "ice3gb_create",
    "ice3gb_destroy", "ice3gb_last_error", "ice3gb_status", "ice3gb_ice_adjust",
    "ice3gb_sedimentation", "ice3gb_rain_ice", "ice3gb_ice_adjust_host", "ice3gb_rain_ice_host",
    "ice3gb_physics_step", "ice3gb_physics_step_host", "ice3gb_profile_enable", "ice3gb_profile_read",
    "ice3gb_kernel_name", "ice3gb_rain_ice_noalloc", "ice3gb_ice_adjust_vjp",
    "ice3gb_sedimentation_vjp", "ice3gb_mlp_create", "ice3gb_mlp_destroy", "ice3gb_mlp_param_count",
    "ice3gb_mlp_get_params", "ice3gb_mlp_set_params", "ice3gb_mlp_forward", "ice3gb_mlp_forward_layered",
    "ice3gb_mlp_loss_grad",
    "ice3gb_mlp_train_step", "ice3gb_mlp_error", "ice3gb_tc_gemm_bf16", "ice3gb_surrogate_sample",
    "ice3gb_rain_ice_surrogate", "ice3gb_physics_step_surrogate",
)
NOALLOC_MAX_POINTS = 4194304
KERNEL_NAMES = ("ice_adjust", "sedimentation", "rain_ice", "rain_ice_evap_fixup", "fog_deposition", "rain_ice_order",
                "ice_adjust_vjp", "sedimentation_vjp", "surrogate_sample", "surrogate_mlp", "rain_ice_surrogate",
                "rain_ice_precip_fraction")

_lib: Optional[ctypes.CDLL] = None


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load libice3gb.so (built by build.py) and declare the signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            f"{path} not found: build the CUDA library first "
            "(python -c 'import __graft_entry__ as g; g.build()' at the repository root)")
    lib = ctypes.CDLL(path)
    lib.ice3gb_version.restype = ctypes.c_int
    lib.ice3gb_constant_count.restype = ctypes.c_int
    lib.ice3gb_constant_name.restype = ctypes.c_char_p
    lib.ice3gb_constant_name.argtypes = [ctypes.c_int]
    lib.ice3gb_create.argtypes = [ctypes.POINTER(Ice3gbConstants), ctypes.POINTER(Ice3gbLuts),
                                  ctypes.POINTER(ctypes.c_void_p)]
    lib.ice3gb_destroy.argtypes = [P]
    lib.ice3gb_last_error.argtypes = [P, ctypes.c_char_p, ctypes.c_size_t]
    lib.ice3gb_status.argtypes = [P, P, ctypes.POINTER(ctypes.c_uint32)]
    lib.ice3gb_ice_adjust.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                      ctypes.POINTER(IceAdjustFields), P]
    lib.ice3gb_ice_adjust_host.argtypes = lib.ice3gb_ice_adjust.argtypes
    lib.ice3gb_sedimentation.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                         ctypes.POINTER(SedimentationFields), P]
    lib.ice3gb_rain_ice.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                    ctypes.POINTER(RainIceOptions), ctypes.POINTER(RainIceFields), P]
    lib.ice3gb_rain_ice_host.argtypes = lib.ice3gb_rain_ice.argtypes
    lib.ice3gb_rain_ice_noalloc.argtypes = lib.ice3gb_rain_ice.argtypes
    lib.ice3gb_rain_ice_noalloc.restype = ctypes.c_int
    lib.ice3gb_physics_step.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                        ctypes.POINTER(RainIceOptions), ctypes.POINTER(StepFields), P]
    lib.ice3gb_physics_step_host.argtypes = lib.ice3gb_physics_step.argtypes
    lib.ice3gb_ice_adjust_vjp.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                          ctypes.POINTER(IceAdjustFields), ctypes.POINTER(IceAdjustCotangents),
                                          ctypes.POINTER(IceAdjustGradients), P]
    lib.ice3gb_ice_adjust_vjp.restype = ctypes.c_int
    lib.ice3gb_sedimentation_vjp.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                             ctypes.POINTER(SedimentationFields),
                                             ctypes.POINTER(SedimentationCotangents),
                                             ctypes.POINTER(SedimentationGradients), P]
    lib.ice3gb_sedimentation_vjp.restype = ctypes.c_int
    lib.ice3gb_profile_enable.argtypes = [P, ctypes.c_int]
    lib.ice3gb_profile_enable.restype = ctypes.c_int
    lib.ice3gb_profile_read.argtypes = [P, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)]
    lib.ice3gb_profile_read.restype = ctypes.c_int
    F = ctypes.POINTER(ctypes.c_float)
    I64 = ctypes.c_int64
    lib.ice3gb_mlp_create.argtypes = [ctypes.POINTER(MlpShape), ctypes.c_uint64, ctypes.POINTER(ctypes.c_void_p)]
    lib.ice3gb_mlp_destroy.argtypes = [P]
    lib.ice3gb_mlp_param_count.argtypes = [P]
    lib.ice3gb_mlp_param_count.restype = I64
    lib.ice3gb_mlp_get_params.argtypes = [P, F]
    lib.ice3gb_mlp_set_params.argtypes = [P, F]
    lib.ice3gb_mlp_forward.argtypes = [P, ctypes.c_int, P, P, P]
    lib.ice3gb_mlp_forward_layered.argtypes = [P, ctypes.c_int, P, P, P]
    lib.ice3gb_mlp_loss_grad.argtypes = [P, ctypes.c_int, P, P, P, P, P]
    lib.ice3gb_mlp_train_step.argtypes = [P, ctypes.c_int, P, P, ctypes.c_float, P, P]
    lib.ice3gb_mlp_error.argtypes = [P]
    lib.ice3gb_tc_gemm_bf16.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, P, I64, I64, P, I64, I64, P, I64,
                                        P, P]
    for name in ("ice3gb_mlp_create", "ice3gb_mlp_destroy", "ice3gb_mlp_get_params", "ice3gb_mlp_set_params",
                 "ice3gb_mlp_forward", "ice3gb_mlp_forward_layered", "ice3gb_mlp_loss_grad", "ice3gb_mlp_train_step", "ice3gb_mlp_error",
                 "ice3gb_tc_gemm_bf16"):
        getattr(lib, name).restype = ctypes.c_int
    NP = ctypes.POINTER(SurrogateNorm)
    U64P = ctypes.POINTER(ctypes.c_uint64)
    lib.ice3gb_surrogate_sample.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                            ctypes.POINTER(RainIceFields), NP, I64, P, P, P, P, P, P]
    lib.ice3gb_rain_ice_surrogate.argtypes = [P, P, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                              ctypes.POINTER(RainIceOptions), ctypes.POINTER(RainIceFields), NP,
                                              U64P, P]
    lib.ice3gb_physics_step_surrogate.argtypes = [P, P, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                                  ctypes.POINTER(RainIceOptions), ctypes.POINTER(StepFields), NP,
                                                  U64P, P]
    for name in ("ice3gb_surrogate_sample", "ice3gb_rain_ice_surrogate", "ice3gb_physics_step_surrogate"):
        getattr(lib, name).restype = ctypes.c_int
    lib.ice3gb_kernel_name.argtypes = [ctypes.c_int]
    lib.ice3gb_kernel_name.restype = ctypes.c_char_p
    for name in ("ice3gb_physics_step", "ice3gb_physics_step_host", "ice3gb_create", "ice3gb_destroy", "ice3gb_last_error", "ice3gb_status",
                 "ice3gb_ice_adjust", "ice3gb_sedimentation", "ice3gb_rain_ice",
                 "ice3gb_ice_adjust_host", "ice3gb_rain_ice_host"):
        getattr(lib, name).restype = ctypes.c_int
    _lib = lib
    return lib


class Ice3gbError(RuntimeError):
    pass


def check(rc: int, handle=None, what: str = "") -> None:
    if rc == ICE3GB_OK:
        return
    lib = load()
    buf = ctypes.create_string_buffer(512)
    lib.ice3gb_last_error(handle, buf, len(buf))
    raise Ice3gbError(f"{what}: {ERRORS.get(rc, rc)}: {buf.value.decode(errors='replace')}")
