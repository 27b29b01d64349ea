"""Float comparisons with the semantics of the `approx` crate used by the
reference's tests (assert_ulps_eq / assert_relative_eq)."""
import struct


def _ordered(x: float) -> int:
    i = struct.unpack("<q", struct.pack("<d", x))[0]
    return i if i >= 0 else -(i & 0x7FFFFFFFFFFFFFFF)


def ulps_eq(a: float, b: float, max_ulps: int = 4, epsilon: float = 2.220446049250313e-16) -> bool:
    if abs(a - b) <= epsilon:
        return True
    if (a < 0) != (b < 0):
        return False
    return abs(_ordered(a) - _ordered(b)) <= max_ulps


def relative_eq(a: float, b: float, epsilon: float = 2.220446049250313e-16,
                max_relative: float = 2.220446049250313e-16) -> bool:
    if a == b:
        return True
    diff = abs(a - b)
    if diff <= epsilon:
        return True
    return diff <= max(abs(a), abs(b)) * max_relative


def rust_round_at(x: float, decimal: int) -> float:
    """RoundAt::round_at of tests/nist-lj.rs:22-30: (x * 10^d).round() / 10^d,
    with f64::round rounding half away from zero."""
    import math
    factor = 10.0 ** decimal
    y = x * factor
    r = math.floor(abs(y))
    if abs(y) - r >= 0.5:
        r += 1.0
    return math.copysign(r, y) / factor
