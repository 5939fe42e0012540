"""Rounding identities the FP32 kernels rely on, checked on the host with IEEE arithmetic
(numpy, no flush to zero).

* The FP32 state transfers form the velocity phi - psi and psi = phi - v with the FP32
  subtraction where the host rows are FP32.  The FP64 difference of two floats rounded once
  to FP32 is the same value: double rounding through 53 bits is innocuous for a sum of two
  24-bit numbers (53 >= 2 * 24 + 2).
* The unwritten cells of the merged update take x + (-v) in place of x - v: IEEE
  subtraction is addition of the negated operand, signs of zero included.
* The skewed strip forms the Laplacian from differences: (n - x) + (sv - x) as
  (n - x) - (x - sv), and (e - x) + (w - x) as (e - x) - (x - w), since round-to-nearest
  is symmetric (sv - x == -(x - sv))."""
import numpy as np

F32 = np.float32


def _pairs(n, seed):
    rng = np.random.default_rng(seed)
    parts = [
        rng.standard_normal((n, 2)),
        rng.standard_normal((n, 2)) * np.exp(rng.uniform(-85, 85, (n, 2))),   # wide exponent gaps
        rng.uniform(-1, 1, (n, 2)) * 1.2e-38,                                   # around the subnormals
        rng.uniform(-3.4e38, 3.4e38, (n, 2)),                                   # overflowing differences
    ]
    ab = np.concatenate(parts).astype(F32)
    tiny = F32(1.4e-45)
    special = np.array([[0.0, -0.0], [-0.0, 0.0], [0.0, 0.0], [-0.0, -0.0], [tiny, -tiny], [tiny, tiny],
                        [3.0e38, -3.0e38], [1.0, 5.9604645e-08], [16777217.0, 1.0], [1e30, 1e-30]], F32)
    ab = np.concatenate([ab, special])
    return ab[:, 0].copy(), ab[:, 1].copy()


def _bits(x):
    return x.view(np.uint32)


def test_fp32_subtraction_equals_rounded_fp64_difference():
    a, b = _pairs(200_000, 1)
    with np.errstate(over="ignore", invalid="ignore"):
        direct = a - b
        via64 = (a.astype(np.float64) - b.astype(np.float64)).astype(F32)
    assert np.array_equal(_bits(direct), _bits(via64))


def test_round_trip_of_the_velocity_form():
    """psi -> v = phi - psi -> psi' = phi - v: the same value whichever way it is formed."""
    a, b = _pairs(100_000, 2)
    with np.errstate(over="ignore", invalid="ignore"):
        v32 = a - b
        v64 = (a.astype(np.float64) - b.astype(np.float64)).astype(F32)
        p32 = a - v32
        p64 = (a.astype(np.float64) - v64.astype(np.float64)).astype(F32)
    assert np.array_equal(_bits(p32), _bits(p64))


def test_subtraction_is_addition_of_the_negation():
    a, b = _pairs(100_000, 3)
    with np.errstate(over="ignore", invalid="ignore"):
        assert np.array_equal(_bits(a - b), _bits(a + (-b)))


def test_laplacian_differences():
    rng = np.random.default_rng(4)
    x, n, s, e, w = (rng.standard_normal(300_000).astype(F32) * F32(10) ** rng.integers(-3, 4, 300_000).astype(F32)
                     for _ in range(5))
    assert np.array_equal(_bits((n - x) + (s - x)), _bits((n - x) - (x - s)))
    assert np.array_equal(_bits((e - x) + (w - x)), _bits((e - x) - (x - w)))
