"""The lower bound behind the BF16-screened k-means++ rounds, checked on the CPU.

A screened round leaves row i alone when a lower bound of the new center's FP32 distance
(the update's sequential fmaf sum) exceeds the row's current distance.  The bound is built
from A, an FP32 sum of squared differences between the row's BF16 copy and the center:
    v >= (A (1 - g) - 2^-7 ||x|| sqrt(A (1 + 2 g)) - 3 2^-16 ||x||^2 - slack) (1 - g),
g = (d + 2) 2^-24 / (1 - (d + 2) 2^-24), slack the subnormal entries' terms.  The kernel
evaluates it in FP32 with every rounding directed against it; here it is evaluated in FP64
(tighter than the kernel's) and must never exceed the FP32 distance, over random rows,
rows next to the center, large and tiny magnitudes and subnormal entries.
"""
import numpy as np
import pytest


def _bf16(x):
    """float32 -> bfloat16 (round to nearest even), returned as float32."""
    b = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    lsb = (b >> 16) & 1
    r = ((b + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def _fp32_seq_dist(x, c):
    """The update's FP32 distance: df = fl(c - x), acc = fmaf(df, df, acc) in column order
    (the product of two floats is exact in FP64, the sum rounded once to float32)."""
    acc = np.float32(0.0)
    for cj, xj in zip(c, x):
        df = np.float64(np.float32(cj - xj))
        acc = np.float32(np.float64(acc) + df * df)
    return float(acc)


def _screen_bound(x, c):
    d = x.size
    g = (d + 2) * 2.0 ** -24 / (1.0 - (d + 2) * 2.0 ** -24)
    xb = _bf16(x)
    # A: any FP32 order (here: products rounded, then summed left to right)
    A = np.float32(0.0)
    for cj, xj in zip(c, xb):
        df = np.float32(xj - cj)
        A = np.float32(A + np.float32(df * df))
    A = float(A)
    xn = float(np.sqrt(np.sum(np.asarray(x, np.float64) ** 2)))
    sq = np.sqrt(A * (1 + 2 * g))
    slack = sq * 2.0 ** -129 + xn * 2.0 ** -135 + 2.0 ** -140
    slo = A * (1 - g) - 2.0 ** -7 * xn * sq - 3 * 2.0 ** -16 * xn * xn - slack
    return max(slo, 0.0) * (1 - g)


@pytest.mark.parametrize("d", [16, 32, 64, 128])
def test_screen_bound_never_exceeds_fp32_distance(d):
    rng = np.random.default_rng(d)
    worst = 0.0
    for trial in range(300):
        kind = trial % 6
        if kind == 0:       # independent rows and centers
            x = rng.normal(size=d).astype(np.float32)
            c = rng.normal(size=d).astype(np.float32)
        elif kind == 1:     # a row next to the center (the settled / unsettled border)
            c = rng.normal(size=d).astype(np.float32) * 10
            x = (c + rng.normal(size=d) * 1e-3).astype(np.float32)
        elif kind == 2:     # large magnitudes
            x = (rng.normal(size=d) * 1e18).astype(np.float32)
            c = (rng.normal(size=d) * 1e18).astype(np.float32)
        elif kind == 3:     # tiny magnitudes with subnormal entries
            x = (rng.normal(size=d) * 1e-39).astype(np.float32)
            c = (rng.normal(size=d) * 1e-39).astype(np.float32)
        elif kind == 4:     # a shared offset much larger than the differences
            off = rng.normal(size=d) * 1e4
            x = (off + rng.normal(size=d)).astype(np.float32)
            c = (off + rng.normal(size=d)).astype(np.float32)
        else:               # mixed scales per column
            s = 10.0 ** rng.integers(-20, 20, size=d)
            x = (rng.normal(size=d) * s).astype(np.float32)
            c = (rng.normal(size=d) * s).astype(np.float32)
        with np.errstate(over="ignore", under="ignore"):  # FP32 overflow: such rows are skipped
            v = _fp32_seq_dist(x, c)
            if not np.isfinite(v):
                continue
            lo = _screen_bound(x, c)
        assert lo <= v, (d, trial, lo, v)
        if v > 0:
            worst = max(worst, lo / v)
    # and it is not vacuous: for ordinary rows the bound is within a few percent of v
    assert worst > 0.9


def test_bf16_unit_roundoff_is_two_to_minus_eight():
    """BF16 keeps an 8-bit significand, so round to nearest errs by up to 2^-8 of |x| (not
    2^-9): 1 + 2^-8 lies halfway between 1 and 1 + 2^-7 and rounds (to even) to 1.  The
    tensor-core certificate's per-operand u and the k-means++ screen both use 2^-8; a product
    of two such operands errs by 2u + u^2 of |x c|, which the 2^-9 figure would not cover."""
    x = np.full(64, 1.0 + 2.0 ** -8, np.float32)
    xb = _bf16(x)
    assert np.all(xb == 1.0)
    rel = np.abs(xb.astype(np.float64) - x) / x
    assert np.all(rel <= 2.0 ** -8) and np.all(rel > 2.0 ** -9)
    # the dot product of the BF16 copies against the exact one
    exact = float(np.dot(x.astype(np.float64), x.astype(np.float64)))
    approx = float(np.dot(xb.astype(np.float64), xb.astype(np.float64)))
    nx = float(np.linalg.norm(x.astype(np.float64)))
    err = abs(approx - exact)
    u8, u9 = 2.0 ** -8, 2.0 ** -9
    assert err <= (2 * u8 + u8 * u8) * nx * nx
    assert err > (2 * u9 + u9 * u9) * nx * nx
    # random operands stay inside the 2^-8 bound
    rng = np.random.default_rng(3)
    for _ in range(200):
        a = (rng.normal(size=128) * 10.0 ** rng.integers(-3, 4)).astype(np.float32)
        b = (rng.normal(size=128) * 10.0 ** rng.integers(-3, 4)).astype(np.float32)
        ex = float(np.dot(a.astype(np.float64), b.astype(np.float64)))
        ap = float(np.dot(_bf16(a).astype(np.float64), _bf16(b).astype(np.float64)))
        bound = (2 * u8 + u8 * u8) * float(np.abs(a.astype(np.float64)) @ np.abs(b.astype(np.float64)))
        assert abs(ap - ex) <= bound * (1 + 1e-12)
