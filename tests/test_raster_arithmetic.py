"""The float arguments the camera raster's exactness rests on, checked on the
CPU with NumPy float32 (every operation rounded once, as the kernels compile
without FMA contraction; a fused multiply-add is emulated exactly).

* step_t (csrc/raster.cu): t = i / n from RN(1/n) with one FMA correction equals
  the correctly rounded quotient for every 0 <= i <= n <= kMaxSteps (96).
* mix at the ends of a segment (the shared-endpoint drop in raster_camera):
  mix(a, b, 1) and mix(b, c, 0) both give b when a and c are finite.
* approx_depth (the division-free depth pre-test) stays within 5 units of
  quantize_depth.
* sqrt_bound: sqrt_rn(x) <= r exactly when x <= sqrt_bound(r).
"""
from fractions import Fraction

import numpy as np

F = np.float32
K_MAX_STEPS = 96


def _rn32(x: Fraction) -> np.float32:
    """x rounded to the nearest float32 (ties to even), for finite normal results."""
    f = F(float(x))  # nearest double, then nearest float
    # repair the rare double rounding: pick the float nearest to x exactly
    lo, hi = np.nextafter(f, F(-np.inf)), np.nextafter(f, F(np.inf))
    best = min((lo, f, hi), key=lambda c: (abs(Fraction(float(c)) - x), int(np.frombuffer(c.tobytes(), np.uint32)[0]) & 1))
    return F(best)


def _fma32(a, b, c) -> np.float32:
    return _rn32(Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c)))


def _mixf(a, b, t):
    """mixf (hg_device.cuh): a * (1 - t) + b * t, each operation rounded."""
    a, b, t = F(a), F(b), F(t)
    return F(F(a * F(F(1) - t)) + F(b * t))


def test_step_t_equals_the_correctly_rounded_quotient():
    for n in range(1, K_MAX_STEPS + 1):
        fn = F(n)
        rcp = _rn32(Fraction(1, n))
        for i in range(0, n + 1):
            fi = F(i)
            q0 = F(fi * rcp)
            rem = _fma32(-q0, fn, fi)
            t = _fma32(rem, rcp, q0)
            assert t == _rn32(Fraction(i, n)), (i, n)


def test_mix_ends_give_the_shared_point():
    rng = np.random.default_rng(7)
    vals = np.concatenate([
        rng.normal(0, 1, 4000), rng.normal(0, 1e4, 4000), rng.uniform(-3, 3, 4000) * 10.0 ** rng.integers(-30, 30, 4000),
        [0.0, -0.0, 1e-40, -1e-40, 3.0e38, -3.0e38],
    ]).astype(F)
    a, b, c = rng.choice(vals, 20000), rng.choice(vals, 20000), rng.choice(vals, 20000)
    with np.errstate(over="ignore", invalid="ignore"):
        end_j = F(a * F(F(1) - F(1))) + F(b * F(1))     # segment j at t = 1
        start_k = F(b * F(F(1) - F(0))) + F(c * F(0))   # segment j + 1 at t = 0
    # equal as values (a signed zero may differ, which no integer output sees)
    assert np.all(end_j == b) and np.all(start_k == b)
    # a non-finite neighbour breaks it, which is why the drop needs finite points
    with np.errstate(invalid="ignore"):
        assert np.isnan(_mixf(np.inf, 1.0, 1.0))


def _quantize_depth(dist, near, far):
    q = np.clip(F(F(dist - near) / np.maximum(F(far - near), F(1e-3))), F(0), F(1))
    r = F(q * F(16777214.0)).astype(np.uint32)
    return np.minimum(r, np.uint32(0x00FFFFFE))


def _approx_depth(dist, near, inv_range):
    with np.errstate(invalid="ignore"):
        q = np.clip(F(F(dist - near) * inv_range), F(0), F(1))
    r = F(q * F(16777214.0)).astype(np.uint32)
    return np.minimum(r, np.uint32(0x00FFFFFE))


def test_approx_depth_within_five_units_of_quantize_depth():
    rng = np.random.default_rng(11)
    for near, far in ((0.1, 1000.0), (0.01, 50.0), (1.0, 5000.0), (0.5, 0.9)):
        near, far = F(near), F(far)
        inv_range = F(F(1) / np.maximum(F(far - near), F(1e-3)))
        dist = rng.uniform(float(near) - 1.0, float(far) + 1.0, 200000).astype(F)
        exact = _quantize_depth(dist, near, far).astype(np.int64)
        approx = _approx_depth(dist, near, inv_range).astype(np.int64)
        assert np.max(np.abs(exact - approx)) <= 5


def _sqrt_bound(r):
    """sqrt_bound (csrc/raster.cu, csrc/filter.cu): the largest x with sqrt_rn(x) <= r."""
    r = F(r)
    x = F(r * r)
    for _ in range(8):
        if not np.sqrt(x) > r:
            break
        x = np.nextafter(x, F(0))
    for _ in range(8):
        up = np.nextafter(x, F(np.inf))
        if not np.sqrt(up) <= r:
            break
        x = up
    return x


def test_sqrt_bound_decides_like_the_square_root():
    rng = np.random.default_rng(3)
    for r in [0.025, 0.05, 0.1, 0.25, 0.5, 0.75, 1.0] + list(rng.uniform(0.02, 2.0, 50)):
        r = F(r)
        x = _sqrt_bound(r)
        assert np.sqrt(x) <= r
        assert np.sqrt(np.nextafter(x, F(np.inf))) > r
        d = (x * (1 + rng.uniform(-1e-5, 1e-5, 20000))).astype(F)
        assert np.array_equal(np.sqrt(d) <= r, d <= x)
