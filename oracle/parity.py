"""Parity criteria used by the GPU tests and the smoke check.

TEST INFRASTRUCTURE ONLY (checker side, with the oracle).
"""
import numpy as np


def sensitivity(fn, inputs, rel=1e-13, trials=3, seed=0):
    """Pointwise spread of an oracle function under random relative
    perturbations of its float64 inputs (|delta| <= rel = 1e-13, ten times the
    ~1e-14 relative accuracy of the device's reformulated transcendentals).
    The spread measures how much the reference computation itself moves under
    rounding-size changes: differences of nearly equal terms and the
    rounding-decided sub-step passes of the ICE4 time splitting.
    `fn(inputs) -> dict`."""
    rng = np.random.default_rng(seed)
    base = fn(inputs)
    spread = {k: np.zeros_like(np.asarray(v, dtype=np.float64)) for k, v in base.items()}
    for _ in range(trials):
        pert = {}
        for k, v in inputs.items():
            a = np.asarray(v)
            pert[k] = a * (1.0 + rel * rng.uniform(-1, 1, a.shape)) if a.dtype == np.float64 else a
        other = fn(pert)
        for k in spread:
            d = np.abs(np.asarray(other[k], dtype=np.float64) - np.asarray(base[k], dtype=np.float64))
            spread[k] = np.maximum(spread[k], np.nan_to_num(d, nan=0.0))
    return base, spread


def assert_parity(got, ref, spread, name, tol=1e-10, floor_frac=1e-5, max_frac_conditioned=0.01, scale=None,
                  alts=()):
    """Parity of a device field against the oracle.

    Every point must satisfy |got-ref| <= tol*max(|ref|, scale, floor) + 4*spread,
    (`scale`, optional, is the magnitude of the terms the value is a sum of),
    where `spread` is the oracle's own response to ~1e-14 input perturbations
    (points whose value comes from cancellation); at most `max_frac_conditioned`
    of the points may need the spread term, and NaN/inf must match exactly.
    `alts`: the oracle's outputs with other outcomes of its rounding-decided
    branches (the depletion ties of the sub-stepping); a point that meets
    tol*max(|alt|, scale, floor) for one of them needs no spread.

    Returns how the points met the bound (see `allowance_stats`)."""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    fg, fr = np.isfinite(got), np.isfinite(ref)
    assert np.array_equal(fg, fr), f"{name}: non-finite values differ"
    g, r, s = got[fr], ref[fr], np.asarray(spread, dtype=np.float64)[fr]
    rms = float(np.sqrt(np.mean(r * r))) if r.size else 0.0
    sc = None if scale is None else np.asarray(scale, dtype=np.float64)[fr]
    mag = np.abs(r) if sc is None else np.maximum(np.abs(r), sc)
    base = tol * np.maximum(mag, floor_frac * rms)
    d = np.abs(g - r)
    alt_ok = np.zeros(d.shape, dtype=bool)
    for a in alts:
        a = np.asarray(a, dtype=np.float64)[fr]
        amag = np.abs(a) if sc is None else np.maximum(np.abs(a), sc)
        alt_ok |= np.abs(g - a) <= tol * np.maximum(amag, floor_frac * rms)
    ok = (d <= base) | alt_ok
    assert np.all(ok | (d <= base + 4.0 * s)), (
        f"{name}: {int(np.sum(~ok & (d > base + 4 * s)))} points beyond tolerance, worst rel "
        f"{float(np.max(np.where(ok, 0.0, d) / np.maximum(np.abs(r), floor_frac * rms + 1e-300))):.3e}")
    frac = 1.0 - float(np.mean(ok)) if r.size else 0.0
    assert frac <= max_frac_conditioned, f"{name}: {frac:.2%} of points need the conditioning allowance"
    return allowance_stats(d, r, base, tol, floor_frac * rms, alt_ok)


def allowance_stats(d, r, base, tol, floor, alt_ok=None):
    """How the points of one field met the parity bound:
    n: finite points compared;
    n_scale: points within tol of the operand scale but not of their own
        magnitude (values that are sums of larger terms);
    n_alt: points within tol of another outcome of the oracle's
        rounding-decided branches (and not of the first);
    n_spread: points that needed the oracle's own conditioning spread;
    worst_rel: max |got-ref| / max(|ref|, floor) over the points matched
        without an alternative outcome;
    worst_excess: max |got-ref| / (tol max(|ref|, scale, floor)) over the
        points that needed the spread (0 when none did)."""
    if alt_ok is None:
        alt_ok = np.zeros(d.shape, dtype=bool)
    own = tol * np.maximum(np.abs(r), floor)
    n_scale = int(np.sum((d > own) & (d <= base)))
    n_alt = int(np.sum((d > base) & alt_ok))
    over = (d > base) & ~alt_ok
    n_spread = int(np.sum(over))
    rel = np.where(alt_ok & (d > base), 0.0, d) / np.maximum(np.abs(r), floor + 1e-300)
    worst_rel = float(np.max(rel)) if d.size else 0.0
    worst_excess = float(np.max(d[over] / np.maximum(base[over], 1e-300))) if n_spread else 0.0
    return {"n": int(d.size), "n_scale": n_scale, "n_alt": n_alt, "n_spread": n_spread, "worst_rel": worst_rel,
            "worst_excess": worst_excess}
