"""ice_adjust on the GPU: parity with the reference JAX golden vectors and with
the oracle, edge cases, properties at the full 1024x1024x90 size."""
import numpy as np
import pytest
import torch

from conftest import assert_parity, load_golden, rel_err, sensitivity
from helpers import TOL

pytestmark = pytest.mark.gpu

DT = 50.0
NAMES = ("t", "rv_out", "rc_out", "ri_out", "cldfr", "hlc_hrc", "hlc_hcf", "hli_hri", "hli_hcf", "cph", "lv", "ls",
         "rvs", "rcs", "ris", "ths")
ARGS = ("sigqsat", "pabs", "sigs", "th", "exn", "exn_ref", "rho_dry_ref", "rv", "rc", "ri", "rr", "rs", "rg",
        "cf_mf", "rc_mf", "ri_mf", "rvs", "rcs", "ris", "ths")


@pytest.fixture(scope="module")
def ia():
    from ice3gb import IceAdjust
    return IceAdjust()


def _dev(st):
    return {k: torch.as_tensor(np.ascontiguousarray(st[k])).cuda() for k in ARGS}


def _spread(table, st):
    import oracle
    return sensitivity(lambda x: oracle.ice_adjust(table, x, DT), {k: np.asarray(st[k]) for k in ARGS})


@pytest.mark.parametrize("case", ["ia_std", "ia_mf"])
def test_matches_reference_jax_golden(ia, case):
    """Device output vs the reference JAX outputs (golden vectors)."""
    g = load_golden(case)
    st = {k[3:]: v for k, v in g.items() if k.startswith("in_")}
    out = ia(**_dev(st), timestep=DT)
    torch.cuda.synchronize()
    _, spread = _spread(ia.table, st)
    for name, o in zip(NAMES, out):
        assert_parity(o.cpu().numpy(), g[f"out_{name}"], spread[name], f"{case}/{name}")


def test_matches_oracle_config0(ia):
    """64x64 columns x 90 levels (the ice_adjust workload size) vs the oracle."""
    from ice3gb.state import make_state
    st = {k: v.numpy() for k, v in make_state(64 * 64, 90, seed=7).items()}
    ref, spread = _spread(ia.table, st)
    out = ia(**_dev(st), timestep=DT)
    for name, o in zip(NAMES, out):
        assert_parity(o.cpu().numpy(), ref[name], spread[name], name)


def test_host_entry_point_equals_device(ia):
    from ice3gb.state import make_state
    st = {k: v.numpy() for k, v in make_state(333, 7, seed=5, precip=True).items()}
    dev = ia(**_dev(st), timestep=DT)
    host = ia(**{k: st[k] for k in ARGS}, timestep=DT)   # numpy -> ice3gb_ice_adjust_host
    for name, d, h in zip(NAMES, dev, host):
        assert isinstance(h, np.ndarray)
        np.testing.assert_array_equal(d.cpu().numpy(), h, err_msg=name)


def test_odd_size_and_unaligned_fields(ia):
    """Odd point count (scalar path) and 8-byte-offset views (unaligned for LDG.128)."""
    import oracle
    from ice3gb.state import make_state
    st = {k: v.numpy() for k, v in make_state(37, 11, seed=9, precip=True).items()}
    ref, spread = _spread(ia.table, st)
    big = {k: torch.zeros(st[k].size + 1, dtype=torch.float64, device="cuda") for k in ARGS}
    views = {}
    for k in ARGS:
        big[k][1:] = torch.as_tensor(st[k].ravel()).cuda()
        views[k] = big[k][1:].view(st[k].shape)
    out = ia(**views, timestep=DT)
    for name, o in zip(NAMES, out):
        assert_parity(o.cpu().numpy(), ref[name], spread[name], name)


def test_jax_layout_full_sigqsat(ia):
    """(ngpblks, nproma, nflevg) arrays with a full 3-D sigqsat, as IceAdjustJAX takes them."""
    g = load_golden("ia_mf")
    st = {k[3:]: v for k, v in g.items() if k.startswith("in_")}
    jax_layout = {k: np.ascontiguousarray(np.asarray(st[k]).T.reshape(4, 6, 90)) for k in ARGS}
    out = ia(**{k: torch.as_tensor(v).cuda() for k, v in jax_layout.items()}, timestep=DT)
    _, spread = _spread(ia.table, st)
    for name, o in zip(NAMES, out):
        back = o.cpu().numpy().reshape(24, 90).T
        assert_parity(back, g[f"out_{name}"], spread[name], name)


def test_properties_full_size_1024x1024x90(ia):
    """94M points: total water conserved to round-off, bounded cloud fraction,
    finite outputs, bitwise determinism across calls."""
    from ice3gb.state import make_state
    st = make_state(1024 * 1024, 90, seed=1, device="cuda")
    args = {k: st[k] for k in ARGS}
    out = ia(**args, timestep=DT)
    o = dict(zip(NAMES, out))
    before = st["rv"] + st["rc"] + st["ri"]
    after = o["rv_out"] + o["rc_out"] + o["ri_out"]
    assert float(((after - before).abs() / before).max()) < 1e-14
    assert float(o["cldfr"].min()) >= 0.0 and float(o["cldfr"].max()) <= 1.0
    for k, v in o.items():
        assert bool(torch.isfinite(v).all()), k
    out2 = ia(**args, timestep=DT)
    for a, b in zip(out, out2):
        assert torch.equal(a, b)
    del st, args, out, out2, o
    torch.cuda.empty_cache()
