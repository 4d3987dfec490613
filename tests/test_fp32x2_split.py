"""The double -> FP32x2 split of hyperdeal_gb300/csrc/hd_df.cuh (x2_from_double,
integer operations only), restated with numpy integer arithmetic and checked
on the CPU: hi + lo reproduces the double to 2^-47 relative over the full-
precision range 2^-103 <= |x| < 2^128, to FP32 precision down to 2^-126, and
zeros / tiny values / overflow map to signed zero / infinity."""
import numpy as np


def split(x):
    b = np.asarray(x, dtype=np.float64).view(np.uint64)
    h = (b >> np.uint64(32)).astype(np.uint32)
    l = (b & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    e = (h >> np.uint32(20)) & np.uint32(0x7FF)
    sgn = h & np.uint32(0x80000000)
    with np.errstate(over="ignore"):
        hn = sgn | ((e - np.uint32(896)) << np.uint32(23)) | ((h & np.uint32(0xFFFFF)) << np.uint32(3)) | (l >> np.uint32(29))
        base = sgn | ((e - np.uint32(919)) << np.uint32(23))
        rb = ((l & np.uint32(0x1FFFFFFF)) + np.uint32(32)) >> np.uint32(6)
    with np.errstate(invalid="ignore", over="ignore"):
        lon = (base + rb).view(np.float32) - base.view(np.float32)  # exact (Sterbenz) where used
    normal = (e - np.uint32(897)) <= np.uint32(253)
    full = (e - np.uint32(920)) <= np.uint32(230)
    big = e > np.uint32(1150)
    nan = (e == np.uint32(0x7FF)) & (((h & np.uint32(0xFFFFF)) | l) != 0)
    hb = np.where(normal, hn, np.where(big, sgn | np.uint32(0x7F800000) | np.where(nan, np.uint32(0x400000), np.uint32(0)), sgn))
    hi = hb.astype(np.uint32).view(np.float32)
    lo = np.where(full, lon, np.float32(0.0)).astype(np.float32)
    return hi, lo


def test_full_precision_range():
    rng = np.random.default_rng(0)
    mant = rng.uniform(1.0, 2.0, 20000)
    expo = rng.integers(-103, 128, 20000)
    x = np.ldexp(mant, expo) * rng.choice([-1.0, 1.0], 20000)
    hi, lo = split(x)
    back = hi.astype(np.float64) + lo.astype(np.float64)
    rel = np.abs(back - x) / np.abs(x)
    assert rel.max() <= 2.0 ** -47
    # hi is x truncated to 24 significant bits: same sign, |hi| <= |x|
    assert np.all(np.sign(hi) == np.sign(x)) and np.all(np.abs(hi.astype(np.float64)) <= np.abs(x))


def test_reduced_and_special_ranges():
    x = np.array([0.0, -0.0, 1e-300, -1e-300, 2.0 ** -110, -(2.0 ** -120), 3.0e38, -1e39, 1e300, np.inf, -np.inf, np.nan])
    hi, lo = split(x)
    assert hi[0] == 0 and not np.signbit(hi[0]) and hi[1] == 0 and np.signbit(hi[1])
    assert hi[2] == 0 and hi[3] == 0 and np.signbit(hi[3])
    # 2^-126 <= |x| < 2^-103: FP32 precision, lo = 0
    for i in (4, 5):
        assert lo[i] == 0 and abs(float(hi[i]) - x[i]) <= 2.0 ** -23 * abs(x[i])
    assert abs(float(hi[6]) + float(lo[6]) - x[6]) <= 2.0 ** -47 * x[6]
    assert np.isinf(hi[7]) and hi[7] < 0 and np.isinf(hi[8]) and hi[8] > 0
    assert np.isinf(hi[9]) and np.isinf(hi[10]) and hi[10] < 0 and np.isnan(hi[11])
