"""ice3gb_rain_ice_noalloc: the rain_ice step for callers that cannot
allocate device memory during the call (their GPU memory belongs to their own
pool, or a cap set outside the library limits it).

Calls the entry point through the C ABI, twice in a row, and checks each
result against ice3gb_rain_ice (the allocating entry point: same kernels, so
the results are identical); checks that a grid above the static scratch
(ICE3GB_NOALLOC_MAX_POINTS points) is refused with ICE3GB_ERR_RANGE.
The file is named to be collected last."""
import ctypes

import numpy as np
import pytest
import torch

from conftest import rel_err
from helpers import TOL

pytestmark = pytest.mark.gpu

DT = 50.0
NK = 90


def _fields(st, nij):
    """ABI fields on the device (fresh copies of the in-out fields)."""
    from ice3gb import _abi
    ins = {"exn": "exn", "dzz": "dzz", "rhodref": "rho_dry_ref", "exnref": "exn_ref", "pabs": "pabs",
           "cldfr": "cldfr", "sigs": "sigs", "tht": "th", "rvt": "rv", "rct": "rc", "rrt": "rr", "rit": "ri",
           "rst": "rs", "rgt": "rg", "sea": "sea", "town": "town"}
    io = {"cit": "ci_t", "hlc_hrc": "hlc_hrc", "hlc_hcf": "hlc_hcf", "hli_hri": "hli_hri", "hli_hcf": "hli_hcf",
          "ths": "ths", "rvs": "rvs", "rcs": "rcs", "rrs": "rrs", "ris": "ris", "rss": "rss", "rgs": "rgs"}
    keep = {k: st[v] for k, v in ins.items()}
    keep.update({k: st[v].clone() for k, v in io.items()})
    for k in ("evap3d", "rainfr"):
        keep[k] = torch.empty((NK, nij), dtype=torch.float64, device="cuda")
    for k in ("inprc", "inprr", "inpri", "inprs", "inprg", "indep"):
        keep[k] = torch.empty((nij,), dtype=torch.float64, device="cuda")
    f = _abi.RainIceFields()
    for k, v in keep.items():
        setattr(f, k, ctypes.c_void_p(v.data_ptr()))
    return f, keep


OUTPUTS = ("cit", "ths", "rvs", "rcs", "rrs", "ris", "rss", "rgs", "evap3d", "rainfr", "inprc", "inprr", "inpri",
           "inprs", "inprg", "indep")


@pytest.mark.parametrize("overrides", [{}, {"MRSTEP": 5e-5, "TSTEP_TS": 10.0}])
def test_noalloc_matches_allocating_entry_point_twice(overrides):
    """Also with the MRSTEP / TSTEP_TS time splitting, whose kernels need no
    more scratch than the default ones."""
    from ice3gb import _abi
    from ice3gb.components import Ice3Handle
    from ice3gb.constants import build_table
    from ice3gb.state import make_state

    nij = 64 * 64
    assert nij * NK <= _abi.NOALLOC_MAX_POINTS
    st = make_state(nij, NK, seed=5, precip=True, device="cuda")
    h = Ice3Handle(build_table(table="phyex", overrides=overrides))
    lib = h.lib
    opt = _abi.RainIceOptions(-1, -1, -1, 0, 0)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    f_ref, ref = _fields(st, nij)
    _abi.check(lib.ice3gb_rain_ice(h.h, nij, NK, DT, ctypes.byref(opt), ctypes.byref(f_ref), stream), h.h,
               "ice3gb_rain_ice")
    for call in range(2):
        f, out = _fields(st, nij)
        _abi.check(lib.ice3gb_rain_ice_noalloc(h.h, nij, NK, DT, ctypes.byref(opt), ctypes.byref(f), stream), h.h,
                   f"ice3gb_rain_ice_noalloc (call {call + 1})")
        torch.cuda.synchronize()
        for k in OUTPUTS:
            a, b = out[k].cpu().numpy(), ref[k].cpu().numpy()
            assert rel_err(a, b) <= TOL, f"call {call + 1}: {k}"
            np.testing.assert_array_equal(a, b, err_msg=f"call {call + 1}: {k}")
    assert h.status() == 0


def test_noalloc_refuses_grids_above_its_scratch():
    from ice3gb import _abi
    from ice3gb.components import Ice3Handle
    from ice3gb.constants import build_table

    h = Ice3Handle(build_table(table="phyex"))
    lib = h.lib
    nij = _abi.NOALLOC_MAX_POINTS // NK + 1           # one column too many
    f = _abi.RainIceFields()                          # never dereferenced: refused first
    rc = lib.ice3gb_rain_ice_noalloc(h.h, nij, NK, DT, None, ctypes.byref(f), None)
    assert rc == -8
    buf = ctypes.create_string_buffer(256)
    lib.ice3gb_last_error(h.h, buf, 256)
    assert b"static scratch" in buf.value


def test_noalloc_refuses_time_split_sedimentation():
    """SEDIM = SPLI takes stream-ordered scratch for its sub-stepped mixing
    ratios, which this entry point cannot allocate: ICE3GB_ERR_UNSUPPORTED
    before any launch, and the in-out fields are left as they were."""
    from ice3gb import _abi
    from ice3gb.components import Ice3Handle
    from ice3gb.constants import build_table
    from ice3gb.state import make_state

    nij = 16 * 16
    st = make_state(nij, NK, seed=7, precip=True, device="cuda")
    h = Ice3Handle(build_table(table="phyex", overrides={"SEDIM": 0.0}))
    opt = _abi.RainIceOptions(-1, -1, -1, 0, 0)
    f, out = _fields(st, nij)
    before = out["rrs"].clone()
    rc = h.lib.ice3gb_rain_ice_noalloc(h.h, nij, NK, DT, ctypes.byref(opt), ctypes.byref(f),
                                       ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == -5
    buf = ctypes.create_string_buffer(256)
    h.lib.ice3gb_last_error(h.h, buf, 256)
    assert b"SPLI" in buf.value
    torch.cuda.synchronize()
    assert torch.equal(out["rrs"], before)


def test_noalloc_refuses_ocnd2_before_any_launch():
    """OCND2 takes stream-ordered scratch for its level heights and droplet
    concentrations: ICE3GB_ERR_UNSUPPORTED, and no kernel has run (the
    sedimentation, which comes first by default, has not touched the sources
    nor the surface precipitation)."""
    from ice3gb import _abi
    from ice3gb.components import Ice3Handle
    from ice3gb.constants import build_table
    from ice3gb.state import make_state

    nij = 16 * 16
    st = make_state(nij, NK, seed=7, precip=True, device="cuda")
    h = Ice3Handle(build_table(table="phyex", overrides={"OCND2": 1.0}))
    opt = _abi.RainIceOptions(-1, -1, -1, 0, 0)
    f, out = _fields(st, nij)
    for k in ("ssio", "ssiu", "ifr", "icldfr"):       # never read: the call is refused first
        out[k] = torch.zeros((NK, nij), dtype=torch.float64, device="cuda")
        setattr(f, k, ctypes.c_void_p(out[k].data_ptr()))
    for k in ("inprc", "inprr", "inpri", "inprs", "inprg"):
        out[k].fill_(-1.0)
    before = {k: out[k].clone() for k in ("rcs", "rrs", "ris", "rss", "rgs", "ths", "rvs", "cit", "inprr", "inprs")}
    rc = h.lib.ice3gb_rain_ice_noalloc(h.h, nij, NK, DT, ctypes.byref(opt), ctypes.byref(f),
                                       ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == -5
    buf = ctypes.create_string_buffer(256)
    h.lib.ice3gb_last_error(h.h, buf, 256)
    assert b"OCND2" in buf.value
    torch.cuda.synchronize()
    for k, v in before.items():
        assert torch.equal(out[k], v), k
