"""The arithmetic facts the mixed-precision solves rest on, checked in IEEE
FP32 with numpy (round to nearest, no fused operations; the kernel code
these restate uses only adds, subtracts and explicit fmaf there).

The node-centric solve forms a fiber's displacement difference at either
end as (x_me - x_other) and flips its sign at the fiber's first end; the
fiber-centric solve forms (x_n2 - x_n1) once. The two agree exactly because
TwoSum is exact and rounding to nearest is symmetric: the difference formed
from the other end is the exact negation, so the force vector, summed with
the same sign, has the same bits (up to the sign of an exact zero, which no
later operation can see: nothing divides by it or tests its sign)."""
import numpy as np

f32 = np.float32


def two_sum(a, b):
    s = (a + b).astype(f32)
    bp = (s - a).astype(f32)
    ap = (s - bp).astype(f32)
    e = ((a - ap).astype(f32) + (b - bp).astype(f32)).astype(f32)
    return s, e


def disp_diff(a_hi, a_lo, b_hi, b_lo):
    """du = x_b - x_a from (hi, lo) records, the kernel's disp_diff."""
    d, ed = two_sum(b_hi, (-a_hi).astype(f32))
    return (d + (ed + (b_lo - a_lo).astype(f32)).astype(f32)).astype(f32)


def _records(rng, n, scale):
    hi = (rng.standard_normal(n) * scale).astype(f32)
    lo = (rng.standard_normal(n) * scale * 1e-8).astype(f32)
    return hi, lo


def test_difference_from_the_other_end_is_the_exact_negation():
    """At a fiber's second end the node-centric solve computes exactly the
    fiber-centric expression; at its first end it negates the difference
    formed from there, which must equal the fiber-centric one bit for bit."""
    rng = np.random.default_rng(5)
    for scale in (1e-6, 1e-3, 0.1, 10.0):
        a_hi, a_lo = _records(rng, 200_000, scale)
        b_hi, b_lo = _records(rng, 200_000, scale)
        # nearby ends too (short fibers: heavy cancellation in the hi parts)
        b_hi[::2] = (a_hi[::2] + (rng.standard_normal(100_000) * scale * 1e-5)).astype(f32)
        fwd = disp_diff(a_hi, a_lo, b_hi, b_lo)
        bwd = disp_diff(b_hi, b_lo, a_hi, a_lo)
        assert np.array_equal(fwd, (-bwd).astype(f32))  # == treats -0 and +0 alike


def test_two_sum_is_exact():
    rng = np.random.default_rng(6)
    a = (rng.standard_normal(100_000) * 10.0).astype(f32)
    b = (rng.standard_normal(100_000) * 1e-3).astype(f32)
    s, e = two_sum(a, b)
    exact = a.astype(np.float64) + b.astype(np.float64)  # exact: FP32 sums fit in FP64
    assert np.array_equal(s.astype(np.float64) + e.astype(np.float64), exact)

