"""Accuracy of the kernels' table-driven FP64 exp / exp10 / log
(dwarf-p-ice3_gb300/csrc/fastmath.cuh), host build of the same source,
against 200-bit mpmath values: at most 2 ulp over the ranges the scheme uses
and the IEEE results on special inputs.  The device build runs the same
operations (explicit FMAs, separately rounded adds and multiplies)."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

mp = pytest.importorskip("mpmath")

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def fm(tmp_path_factory):
    out = tmp_path_factory.mktemp("fm") / "libfm_host.so"
    src = os.path.join(HERE, "fastmath_host.cpp")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC", src, "-o", str(out)],
                   check=True)
    lib = ctypes.CDLL(str(out))
    lib.fm_eval.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_long]
    lib.fm_div.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                           ctypes.c_long]

    def ev(fn, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        lib.fm_eval(fn, x.ctypes.data, y.ctypes.data, x.size)
        return y
    ev.lib = lib
    return ev


def ulp_err(got, exact_fn, xs):
    mp.mp.prec = 200
    worst = 0.0
    for g, x in zip(got, xs):
        e = exact_fn(mp.mpf(float(x)))
        ed = float(e)
        if ed == 0.0 or not np.isfinite(ed):
            continue
        u = np.spacing(abs(ed))
        worst = max(worst, float(abs(mp.mpf(float(g)) - e) / u))
    return worst


def test_fexp_within_2ulp(fm):
    rng = np.random.default_rng(1)
    xs = np.concatenate([rng.uniform(-745, 709.7, 3000), rng.uniform(-40, 40, 3000), rng.uniform(-1e-3, 1e-3, 500),
                         rng.uniform(-720, -708, 300), [0.0, -0.0, 1e-300, -1e-300, 1.0, -1.0, 708.0, -708.0]])
    assert ulp_err(fm(0, xs), mp.exp, xs) <= 2.0


def test_fexp10_within_2ulp(fm):
    rng = np.random.default_rng(2)
    xs = np.concatenate([rng.uniform(-300, 300, 3000), rng.uniform(-12, 3, 3000), [0.0, 1.0, -3.5, 2.0]])
    assert ulp_err(fm(1, xs), lambda v: mp.power(10, v), xs) <= 2.0


def test_flog_within_2ulp(fm):
    rng = np.random.default_rng(3)
    xs = np.concatenate([
        10.0 ** rng.uniform(-300, 300, 3000),            # all magnitudes
        rng.uniform(0.99, 1.01, 2000),                  # around 1 (no cancellation allowed)
        rng.uniform(0.5, 2.0, 2000),
        10.0 ** rng.uniform(-320, -308, 200),           # subnormals
        [1.0, 2.0, 0.5, np.sqrt(2.0), 1.0 + 2 ** -52, 1.0 - 2 ** -53, 5e-324, 1.7976931348623157e308]])
    assert ulp_err(fm(2, xs), mp.log, xs) <= 2.0


def test_special_inputs(fm):
    inf, nan = np.inf, np.nan
    e = fm(0, np.array([nan, inf, -inf, 710.0, -746.0, 0.0]))
    assert np.isnan(e[0]) and e[1] == inf and e[2] == 0.0 and e[3] == inf and e[4] == 0.0 and e[5] == 1.0
    e10 = fm(1, np.array([nan, inf, -inf, 309.0, -324.0, 0.0, 2.0]))
    assert np.isnan(e10[0]) and e10[1] == inf and e10[2] == 0.0 and e10[3] == inf and e10[4] == 0.0
    assert e10[5] == 1.0 and e10[6] == 100.0
    lg = fm(2, np.array([nan, inf, 0.0, -0.0, -1.0, 1.0, -inf]))
    assert np.isnan(lg[0]) and lg[1] == inf and lg[2] == -inf and lg[3] == -inf and np.isnan(lg[4])
    assert lg[5] == 0.0 and np.isnan(lg[6])


def test_exp_log_round_trip(fm):
    rng = np.random.default_rng(4)
    x = 10.0 ** rng.uniform(-30, 30, 100000)
    y = fm(0, fm(2, x))
    assert np.max(np.abs(y / x - 1.0)) < 2e-14      # |log x| <= 70: ~70 ulp amplification at most


def test_frcp_within_2ulp(fm):
    rng = np.random.default_rng(5)
    xs = np.concatenate([10.0 ** rng.uniform(-37, 37, 4000), -(10.0 ** rng.uniform(-30, 30, 2000)),
                         rng.uniform(1.0, 2.0, 2000), [1.0, 2.0, 3.0, 0.1, 1e-20, 1e20]])
    assert ulp_err(fm(3, xs), lambda v: 1 / v, xs) <= 1.0
    edge = fm(3, np.array([0.0, -0.0, np.inf, 1e-300, 1e300, np.nan]))
    assert edge[0] == np.inf and edge[1] == -np.inf and edge[2] == 0.0 and np.isnan(edge[5])
    assert edge[3] == 1.0 / 1e-300 and edge[4] == 1.0 / 1e300


def test_fatan_within_2ulp(fm):
    rng = np.random.default_rng(6)
    xs = np.concatenate([rng.uniform(-1, 1, 3000), rng.uniform(-20, 20, 3000), 10.0 ** rng.uniform(-12, 17, 2000),
                         -(10.0 ** rng.uniform(-12, 17, 1000)), [0.0, 1.0, -1.0, 1e-40, 0.5, 2.0, 1.55 * 2.0]])
    assert ulp_err(fm(4, xs), mp.atan, xs) <= 2.0
    edge = fm(4, np.array([np.inf, -np.inf, np.nan, -0.0, 1e300]))
    assert edge[0] == np.pi / 2 and edge[1] == -np.pi / 2 and np.isnan(edge[2]) and edge[3] == 0.0
    assert edge[4] == np.pi / 2


def test_frsqrt_within_1ulp(fm):
    rng = np.random.default_rng(7)
    xs = np.concatenate([10.0 ** rng.uniform(-36, 36, 4000), rng.uniform(1.0, 4.0, 3000),
                         rng.uniform(1e-12, 1e-7, 2000), [1.0, 2.0, 4.0, 0.25, 3.0, 1.718e-5, 2.0 ** 119]])
    assert ulp_err(fm(5, xs), lambda v: 1 / mp.sqrt(v), xs) <= 1.0
    edge = fm(5, np.array([0.0, np.inf, -1.0, np.nan, 1e-300, 1e300]))
    assert edge[0] == np.inf and edge[1] == 0.0 and np.isnan(edge[2]) and np.isnan(edge[3])
    assert edge[4] == 1.0 / np.sqrt(1e-300) and edge[5] == 1.0 / np.sqrt(1e300)


def test_fdiv_rn_is_the_ieee_quotient(fm):
    """fdiv_rn / fdiv_rn2 return the IEEE quotient bit for bit: random
    operands over the whole accepted range and magnitudes of the scheme,
    significands near 1 and 2 (where ulp changes), powers of two, and values
    outside the range (the fallback)."""
    rng = np.random.default_rng(8)
    n = 400000
    a = np.concatenate([10.0 ** rng.uniform(-100, 100, n), rng.uniform(1e6, 3e6, n), -(10.0 ** rng.uniform(-20, 20, n)),
                        np.ldexp(1.0 + rng.integers(0, 64, n) * 2.0 ** -52, rng.integers(-50, 50, n)),
                        np.ldexp(2.0 - rng.integers(1, 64, n) * 2.0 ** -52, rng.integers(-50, 50, n))])
    b = np.concatenate([10.0 ** rng.uniform(-100, 100, n), rng.uniform(900.0, 4000.0, n), 10.0 ** rng.uniform(-20, 20, n),
                        np.ldexp(2.0 - rng.integers(1, 64, n) * 2.0 ** -52, rng.integers(-50, 50, n)),
                        np.ldexp(1.0 + rng.integers(0, 64, n) * 2.0 ** -52, rng.integers(-50, 50, n))])
    a = np.concatenate([a, [1.0, 3.0, 1e300, 1e-300, 0.0, -0.0, np.inf, np.nan, 7.0]])
    b = np.concatenate([b, [4.0, 1.5, 3.0, 7.0, 2.0, 3.0, 5.0, 2.0, 0.0]])
    q, q2 = np.empty_like(a), np.empty_like(a)
    fm.lib.fm_div(0, a.ctypes.data, b.ctypes.data, q.ctypes.data, q2.ctypes.data, a.size)
    with np.errstate(divide="ignore", invalid="ignore"):
        ref = a / b
        ref2 = (2.5 * a) / b
    np.testing.assert_array_equal(q.view(np.uint64), ref.view(np.uint64))
    fm.lib.fm_div(1, a.ctypes.data, b.ctypes.data, q.ctypes.data, q2.ctypes.data, a.size)
    np.testing.assert_array_equal(q.view(np.uint64), ref.view(np.uint64))
    np.testing.assert_array_equal(q2.view(np.uint64), ref2.view(np.uint64))
