"""CPU check of the integer-pipe FP32 <-> FP64 conversions used by the mixed form's
tridiagonal solve (widen / narrow in fen_gb300/csrc/fen_kernels.cuh).

The device functions rewrite IEEE-754 fields with integer operations; this test applies the
same field arithmetic to numpy integers and compares it bit for bit with IEEE casts (exact
widening, round-to-nearest-even narrowing) on normal values, rounding ties, carries into
the exponent and the range edges.  Values outside the handled range take the hardware cast
on the device and are excluded here by the same range test.
"""
import numpy as np


def widen_bits(u):
    u = u.astype(np.uint64)
    hi = (u & 0x80000000) | (((u & 0x7FFFFFFF) >> 3) + 0x38000000)
    lo = (u << 29) & 0xFFFFFFFF
    return (hi << 32) | lo


def narrow_bits(b):
    b = b.astype(np.uint64)
    hi = (b >> 32) & 0xFFFFFFFF
    lo = b & 0xFFFFFFFF
    e = (hi >> 20) & 0x7FF
    ok = (e >= 897) & (e <= 1150)
    f = (hi & 0x80000000) | (((e - 896) & 0xFF) << 23) | ((hi & 0xFFFFF) << 3) | (lo >> 29)
    rem = lo & 0x1FFFFFFF
    up = (rem > 0x10000000) | ((rem == 0x10000000) & ((f & 1) == 1))
    f = (f + up.astype(np.uint64)) & 0xFFFFFFFF
    return f.astype(np.uint32), ok


def test_widen_is_exact():
    rng = np.random.Generator(np.random.PCG64(0))
    x = np.concatenate([rng.standard_normal(200000).astype(np.float32),
                        (rng.standard_normal(20000) * 1e30).astype(np.float32),
                        (rng.standard_normal(20000) * 1e-30).astype(np.float32),
                        np.array([np.finfo(np.float32).max, np.finfo(np.float32).tiny, -1.0, 1.0], np.float32)])
    u = x.view(np.uint32)
    ex = u & 0x7F800000
    normal = (ex != 0) & (ex != 0x7F800000)
    got = widen_bits(u[normal]).view(np.float64)
    assert np.array_equal(got, x[normal].astype(np.float64))


def test_narrow_rounds_to_nearest_even():
    rng = np.random.Generator(np.random.PCG64(1))
    d = np.concatenate([rng.standard_normal(200000), rng.standard_normal(20000) * 1e35,
                        rng.standard_normal(20000) * 1e-35])
    # exact ties and near-ties: float values plus half an FP32 ulp (+- one FP64 ulp)
    f = rng.standard_normal(20000).astype(np.float32)
    half = np.spacing(f.astype(np.float64)) * 0 + np.spacing(np.abs(f)).astype(np.float64) / 2
    ties = f.astype(np.float64) + half
    d = np.concatenate([d, ties, np.nextafter(ties, np.inf), np.nextafter(ties, -np.inf),
                        np.array([3.4028235677973366e38, 3.4028234663852886e38, 1.1754943508222875e-38])])
    bits, ok = narrow_bits(d.view(np.uint64))
    want = d[ok].astype(np.float32)
    assert ok.sum() > 200000
    assert np.array_equal(bits[ok], want.view(np.uint32))
