"""Deterministic inputs for golden vectors and parity tests.

A splitmix64 stream (pure numpy, identical on every machine and numpy
version) so that the digests in golden.json can be recomputed anywhere.
"""
import numpy as np

D = 2048
Q1 = 268369921
Q2 = 249561089
Q = Q1 * Q2
_M = np.uint64(0xFFFFFFFFFFFFFFFF)


def stream(seed: int, count: int) -> np.ndarray:
    """count uint64 values of splitmix64 starting from `seed`."""
    with np.errstate(over="ignore"):
        idx = np.arange(1, count + 1, dtype=np.uint64)
        z = np.uint64(seed) + idx * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def residues(seed: int, lead) -> np.ndarray:
    """Canonical NTT-form array uint32 (*lead, 2, D)."""
    lead = tuple(lead)
    n = int(np.prod(lead, dtype=np.int64)) if lead else 1
    s = stream(seed, n * 2 * D).reshape(n, 2, D)
    out = np.empty_like(s)
    out[:, 0] = s[:, 0] % np.uint64(Q1)
    out[:, 1] = s[:, 1] % np.uint64(Q2)
    return out.astype(np.uint32).reshape(lead + (2, D))


def raw(seed: int, lead) -> np.ndarray:
    """Raw coefficients mod q, uint64 (*lead, D)."""
    lead = tuple(lead)
    n = int(np.prod(lead, dtype=np.int64)) if lead else 1
    return (stream(seed, n * D) % np.uint64(Q)).reshape(lead + (D,))


def bytes_(seed: int, shape) -> np.ndarray:
    n = int(np.prod(shape, dtype=np.int64))
    return (stream(seed, n) & np.uint64(0xFF)).astype(np.uint8).reshape(shape)
