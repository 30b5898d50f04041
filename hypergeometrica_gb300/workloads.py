"""Seeded synthetic operands for tests and benchmarks.

Limbs come from SplitMix64 (Steele, Lea & Flood 2014): value k of the stream
with seed s mixes s + (k+1) * 0x9E3779B97F4A7C15.  Three distributions, as
the benchmark configurations specify:
  uniform  every limb uniform, top limb forced nonzero;
  ones     every limb 0xFFFFFFFFFFFFFFFF (longest carry chains);
  sparse   a limb is nonzero with probability 1/100 (mask from the stream of
           seed s, values from the stream of seed s ^ 0x5DEECE66D), top limb
           forced nonzero.
"""

from __future__ import annotations

import numpy as np

GAMMA = np.uint64(0x9E3779B97F4A7C15)
M1 = np.uint64(0xBF58476D1CE4E5B9)
M2 = np.uint64(0x94D049BB133111EB)
SPARSE_SALT = 0x5DEECE66D


def splitmix64(seed: int, n: int, start: int = 0) -> np.ndarray:
    """Values start .. start+n-1 of the SplitMix64 stream with this seed."""
    with np.errstate(over="ignore"):
        k = np.arange(start + 1, start + n + 1, dtype=np.uint64)
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + k * GAMMA
        z = (z ^ (z >> np.uint64(30))) * M1
        z = (z ^ (z >> np.uint64(27))) * M2
        return z ^ (z >> np.uint64(31))


def limbs(seed: int, n: int, dist: str = "uniform") -> np.ndarray:
    """n little-endian 64-bit limbs of the given distribution."""
    if n == 0:
        return np.zeros(0, dtype=np.uint64)
    if dist == "uniform":
        v = splitmix64(seed, n)
    elif dist == "ones":
        v = np.full(n, 0xFFFFFFFFFFFFFFFF, dtype=np.uint64)
    elif dist == "sparse":
        mask = splitmix64(seed, n) % np.uint64(100) == 0
        v = np.where(mask, splitmix64(seed ^ SPARSE_SALT, n), np.uint64(0)).astype(np.uint64)
    else:
        raise ValueError(f"unknown distribution {dist!r}")
    if v[-1] == 0:
        v[-1] = 1
    return v


def log_uniform_sizes(seed: int, count: int, lo_bits: int, hi_bits: int) -> np.ndarray:
    """count sizes drawn log-uniformly in [2^lo_bits, 2^hi_bits]."""
    u = splitmix64(seed, count).astype(np.float64) / 2.0**64
    return np.floor(2.0 ** (lo_bits + u * (hi_bits - lo_bits))).astype(np.int64)
