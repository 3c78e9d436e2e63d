"""CPU proofs of the kernels' exact-arithmetic shortcuts: a rewritten float
expression that must give the reference expression's IEEE single-precision
result for every input it can receive."""
import numpy as np


def _rn32_exact(hi, lo):
    """Round the exact value hi + lo (float64 pair, |lo| <= ulp(hi) / 2) to
    float32, ties to even."""
    r = hi.astype(np.float32)
    # hi on a float32 midpoint: the sign of lo decides, ties (lo == 0) to even
    up = np.nextafter(r, np.float32(np.inf))
    dn = np.nextafter(r, np.float32(-np.inf))
    mid_up = (r.astype(np.float64) + up.astype(np.float64)) / 2
    mid_dn = (r.astype(np.float64) + dn.astype(np.float64)) / 2
    r = np.where((hi == mid_up) & (lo > 0), up, r)
    r = np.where((hi == mid_dn) & (lo < 0), dn, r)
    return r


def test_depth_quotient_is_the_ieee_division_for_every_u16():
    """depth_m (ss_internal.cuh): RN(d / 1000) for every u16 d (the reference's
    (float)depth / 1000, GPUVoxelGrid.h:306) as q0 = RN(d y), y = RN(1/1000),
    r = fma(-q0, 1000, d), q = fma(r, y, q0)."""
    d = np.arange(65536, dtype=np.float32)
    want = d / np.float32(1000.0)  # IEEE single-precision division
    y = np.float32(1.0e-3)
    assert y == np.float32(1.0) / np.float32(1000.0)
    d64, y64 = d.astype(np.float64), np.float64(y)
    q0 = (d64 * y64).astype(np.float32)  # d y is exact in float64: one rounding
    rem = d64 - q0.astype(np.float64) * 1000.0  # exact in float64 (34-bit product, cancellation)
    r = rem.astype(np.float32)
    assert np.array_equal(r.astype(np.float64), rem)  # the fma's remainder is exact
    p = r.astype(np.float64) * y64  # exact (48-bit product)
    q0d = q0.astype(np.float64)
    hi = q0d + p
    bb = hi - q0d
    lo = (q0d - (hi - bb)) + (p - bb)  # TwoSum: hi + lo == q0 + p exactly
    got = _rn32_exact(hi, lo)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
