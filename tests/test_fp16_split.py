"""Error bounds of the 2xFP16 operand split used by the tensor-core message kernels, on the CPU.

bqa_gb300/csrc/tc_f16x2_d3c16.cuh scales each operand block by 2^k so that its largest
magnitude lies in [2^14, 2^15) (scale_exp, clamped to [-50, 50]), then splits v 2^k = hi + lo
with hi = FP16(v 2^k) and lo = FP16(v 2^k - hi) (round to nearest even, as __float2half_rn),
and the tensor cores accumulate A_lo B_hi + A_hi B_lo + A_hi B_hi in FP32.  numpy's float16
conversion rounds the same way, so the bounds the kernels rely on are checked here:
  * the split residual is below 2^-22 |v 2^k| plus 2^-25 (FP16's subnormal spacing / 2);
  * a 32-term dot product of split operands (lo x lo dropped) is FP32-accurate normwise:
    its error stays below 2^-20 max|a| max|b| (measured about 2^-23), also for blocks whose
    elements span many decades.  The bound is relative to the blocks' largest magnitudes, not
    componentwise: a dot product of elements many decades below the block maximum keeps that
    absolute error (for 12 decades of spread, up to about 2^-16 of sum |a_i b_i|, where an FP32
    dot product would stay near 2^-24 of it).
"""
import numpy as np


def scale_exp(mx):
    """Exponent k with 2^14 <= mx 2^k < 2^15, clamped to [-50, 50]; 0 for mx = 0."""
    if mx == 0:
        return 0
    e = int(np.floor(np.log2(np.float32(mx))))
    return max(-50, min(50, 14 - e))


def split(v):
    """v (float32 array) -> (hi, lo, k) with v 2^k = hi + lo + residual."""
    k = scale_exp(np.abs(v).max())
    vs = (v.astype(np.float64) * 2.0 ** k).astype(np.float32)
    hi = vs.astype(np.float16)
    lo = (vs - hi.astype(np.float32)).astype(np.float16)
    return hi, lo, k, vs


def test_split_residual_bound():
    rng = np.random.default_rng(0)
    for decades in (1, 6, 12, 30):
        v = (rng.normal(size=4096) * 10.0 ** rng.uniform(-decades, 0, size=4096)).astype(np.float32)
        hi, lo, k, vs = split(v)
        assert np.abs(hi.astype(np.float64)).max() < 2.0 ** 15   # no overflow
        res = vs.astype(np.float64) - hi.astype(np.float64) - lo.astype(np.float64)
        assert np.all(np.abs(res) <= 2.0 ** -22 * np.abs(vs) + 2.0 ** -25)


def test_split_dot_products_are_fp32_accurate():
    rng = np.random.default_rng(1)
    for decades in (1, 6, 12):
        for _ in range(50):
            a = (rng.normal(size=32) * 10.0 ** rng.uniform(-decades, 0, size=32)).astype(np.float32)
            b = (rng.normal(size=32) * 10.0 ** rng.uniform(-decades, 0, size=32)).astype(np.float32)
            ah, al, ka, _ = split(a)
            bh, bl, kb, _ = split(b)
            f = lambda x: x.astype(np.float64)
            got = (f(al) @ f(bh) + f(ah) @ f(bl) + f(ah) @ f(bh)) * 2.0 ** -(ka + kb)
            exact = f(a) @ f(b)
            assert abs(got - exact) <= 2.0 ** -20 * np.abs(f(a)).max() * np.abs(f(b)).max()


def test_scale_exponent_clamp():
    assert scale_exp(0.0) == 0
    assert scale_exp(1.0) == 14
    assert scale_exp(2.0 ** 14) == 0
    assert scale_exp(2.0 ** -60) == 50       # tiny blocks sit below [2^14, 2^15) instead
    assert scale_exp(2.0 ** 70) == -50
