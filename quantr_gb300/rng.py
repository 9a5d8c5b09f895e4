"""SplitMix64 streams: the seeded generator of `measure_all` and of the synthetic workloads.

quantr draws shots with `fastrand::f64()` from a thread-local generator that tests reseed with
`fastrand::seed(0)` (tests/grovers.rs:23, 75). Its stream is not reproduced: `seed(s)` resets a
SplitMix64 stream here (Steele, Lea & Flood, OOPSLA 2014), and each `measure_all` takes one
64-bit key from it for the device sampler. Doubles are (x >> 11) * 2^-53 in [0, 1).
"""
from __future__ import annotations

import math

_MASK = (1 << 64) - 1
GOLDEN = 0x9E3779B97F4A7C15


def mix64(z: int) -> int:
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK
    return z ^ (z >> 31)


class SplitMix64:
    def __init__(self, seed: int):
        self.state = seed & _MASK

    def next_u64(self) -> int:
        self.state = (self.state + GOLDEN) & _MASK
        return mix64(self.state)

    def next_f64(self) -> float:
        return (self.next_u64() >> 11) * (1.0 / (1 << 53))

    def uniform(self, lo: float, hi: float) -> float:
        return lo + (hi - lo) * self.next_f64()

    def below(self, n: int) -> int:
        """Uniform integer in [0, n) by rejection-free multiply-shift (bias < 2^-32 for small n)."""
        return (self.next_u64() >> 32) * n >> 32

    def normal(self) -> float:
        """Standard normal by Box-Muller from two draws."""
        u1 = 1.0 - self.next_f64()  # (0, 1]
        u2 = self.next_f64()
        return math.sqrt(-2.0 * math.log(u1)) * math.cos(2.0 * math.pi * u2)


_global = SplitMix64(0)


def seed(s: int) -> None:
    """`fastrand::seed` counterpart for the shot generator."""
    global _global
    _global = SplitMix64(s)


def next_u64() -> int:
    return _global.next_u64()


def next_f64() -> float:
    return _global.next_f64()
