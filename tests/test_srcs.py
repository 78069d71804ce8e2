"""PSRCS (s'r_c'/sigma_s^2, the second-order flux term the Fortran
ICE_ADJUST returns, ice_adjust.F90:360, :468; condensation.F90:566-571,
:638-647): the oracle's SRC_1D table against the reference's
(tests/golden/src_1d.npz), the device code's host build against the
oracle (CPU), and the device kernels (two-point and scalar paths, device
and host buffers) against the oracle (GPU)."""
import ctypes

import numpy as np
import pytest

import test_adjoint_host as H
from conftest import load_golden, rel_err
from helpers import TOL
from test_adjoint_host import lib  # noqa: F401  (host build of the point code, a fixture)

DT = 50.0
# (LSUBG_COND, LAMBDA3): AROME (subgrid condensation, CB), no CB factor, all-or-nothing
CASES = [(1.0, 0.0), (1.0, 1.0), (0.0, 0.0)]


def _table(subg, lam):
    from ice3gb.constants import build_table
    return build_table(table="jax", overrides={"LSUBG_COND": subg, "LAMBDA3": lam})


def test_src_1d_table_matches_reference():
    import oracle
    np.testing.assert_array_equal(oracle.src_1d(), load_golden("src_1d")["SRC_1D"])


@pytest.mark.parametrize("subg,lam", CASES)
def test_host_build_matches_oracle(lib, subg, lam):  # noqa: F811
    import oracle
    t = _table(subg, lam)
    x = H._state(64 * 64, seed=31)
    ref = oracle.ice_adjust(t, x, DT, srcs=True)["srcs"]
    n = x["th"].size
    ins = [np.ascontiguousarray(x[k], dtype=np.float64).ravel() for k in H.IN]
    got = np.empty(n)
    lib.ia_srcs_host(ctypes.byref(t.consts), ctypes.c_double(DT), ctypes.c_long(n), H._ptrs(ins),
                     got.ctypes.data_as(ctypes.c_void_p))
    # q1 is a cancelling difference: last-bit changes move the small
    # table entries by ~1e-16 absolute, hence the field-scale floor of rel_err
    assert rel_err(got, ref.ravel()) <= TOL
    assert np.count_nonzero((ref > 0) & (ref < 1)) > 100 or subg == 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("subg,lam", CASES)
@pytest.mark.parametrize("aligned", [True, False])          # two-point (128-bit) kernel / scalar kernel
def test_device_matches_oracle(subg, lam, aligned):
    import oracle
    import torch
    from ice3gb import IceAdjust
    x = H._state(64 * 64, seed=32)
    ia = IceAdjust()
    ia.table = _table(subg, lam)
    ref = oracle.ice_adjust(ia.table, x, DT, srcs=True)

    def put(v):
        t = torch.as_tensor(v).cuda()
        if aligned:
            return t
        buf = torch.empty(t.numel() + 1, dtype=t.dtype, device="cuda")   # 8-byte offset: not 16-byte aligned
        return buf[1:].view(t.shape).copy_(t)
    dev = {k: put(v) for k, v in x.items()}
    res = ia(**dev, timestep=DT, return_srcs=True)
    assert len(res) == 17
    assert rel_err(res[16].cpu().numpy(), ref["srcs"]) <= TOL
    # the other outputs are unchanged by asking for srcs
    plain = ia(**dev, timestep=DT)
    for a, b in zip(plain, res[:16]):
        assert torch.equal(a, b)
    host = ia(**x, timestep=DT, return_srcs=True)
    np.testing.assert_array_equal(host[16], res[16].cpu().numpy())
