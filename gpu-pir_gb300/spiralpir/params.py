"""Spiral parameters for the GB300 answer path.

The ring (d = 2048) and the two CRT primes are fixed; everything else is a
runtime parameter, unlike the reference, which compiles them in
(gpu-pir/params.cuh:55-74).  A context carries the gadget lengths and the
plaintext/response moduli; each database carries its own (nu1, nu2).
"""
from __future__ import annotations

import dataclasses

D = 2048
Q1 = 268369921
Q2 = 249561089
Q = Q1 * Q2
MOD_BITS = 56


def ceil_log2(x: int) -> int:
    v, p = 0, 1
    while p < x:
        p <<= 1
        v += 1
    return v


def bits_per(t: int) -> int:
    """Digit width of a length-t gadget: ceil(56 / t) (gpu-pir/gadget.cuh:37-39)."""
    return (MOD_BITS + t - 1) // t


@dataclasses.dataclass(frozen=True)
class SpiralParams:
    n: int = 2              # plaintext matrices are n x n
    pt_bits: int = 8        # p = 2^pt_bits
    t_exp_left: int = 8     # expansion gadget, even (first-dimension) branch
    t_exp_right: int = 8    # expansion gadget, odd (GSW-bit) branch
    t_gsw: int = 7          # GSW / folding gadget
    t_conv: int = 4         # Regev->GSW conversion and packing gadget
    q2_bits: int = 22       # response first-row modulus 2^q2_bits

    @property
    def p(self) -> int:
        return 1 << self.pt_bits

    @property
    def T(self) -> int:
        """Number of plaintext polynomials per record (n*n)."""
        return self.n * self.n

    @property
    def record_bytes(self) -> int:
        return self.T * D * ((self.pt_bits + 7) // 8)

    def g(self, nu1: int, nu2: int) -> int:
        return ceil_log2(self.t_gsw * nu2 + (1 << nu1))

    def stop_round(self, nu2: int) -> int:
        return ceil_log2(self.t_gsw * nu2)

    def response_bytes(self) -> int:
        bits = self.n * D * self.q2_bits + self.T * D * (self.pt_bits + 2)
        return (bits + 63) // 64 * 8

    def db_device_bytes(self, nu1: int, nu2: int) -> int:
        """Bytes of the CRT-NTT database image on the device (two 28-bit
        residues, 7 bytes, per coefficient; combo blocks narrower than 8 are
        padded to 8 combo places)."""
        combos = self.T << nu2
        cb = min(combos, 128)
        cbp = (cb + 7) // 8 * 8
        return 2 * D * (combos // cb) * (1 << nu1) * cbp * 7 // 2


@dataclasses.dataclass(frozen=True)
class DbShape:
    nu1: int
    nu2: int

    @property
    def rows(self) -> int:
        return 1 << self.nu1

    @property
    def cols(self) -> int:
        return 1 << self.nu2

    @property
    def num_records(self) -> int:
        return 1 << (self.nu1 + self.nu2)


# Workloads of the answer path (ring d = 2048, q = q1*q2, p = 256, n = 2,
# t_exp = 8, t_gsw = 7, t_conv = 4).
PARAMS = SpiralParams()
SHAPE_8MIB = DbShape(7, 3)      # 1024 records of 8 KiB: 8 MiB plaintext
SHAPE_64MIB = DbShape(8, 5)     # 8192 records: 64 MiB plaintext
SHAPE_1GIB = DbShape(9, 8)      # 2^17 records: 1 GiB plaintext, 7 GiB image on the device
SHAPE_8GIB = DbShape(9, 11)     # 2^20 records: 8 GiB plaintext, 56 GiB image on the device

# The parameters of the reference's golden vectors (gpu-pir/params.cuh:65-71).
FIXTURE_PARAMS = SpiralParams(n=1, pt_bits=8, t_exp_left=8, t_exp_right=8, t_gsw=8, t_conv=4,
                              q2_bits=22)
FIXTURE_SHAPE = DbShape(6, 2)


def delta(p: SpiralParams) -> int:
    return Q // p.p


def human_bytes(b: int) -> str:
    for unit in ("B", "KiB", "MiB", "GiB", "TiB"):
        if b < 1024 or unit == "TiB":
            return f"{b:.0f} {unit}" if unit == "B" else f"{b:.1f} {unit}"
        b /= 1024
    return str(b)


__all__ = [
    "D", "Q1", "Q2", "Q", "MOD_BITS", "SpiralParams", "DbShape", "PARAMS", "SHAPE_8MIB",
    "SHAPE_64MIB", "SHAPE_1GIB", "SHAPE_8GIB", "FIXTURE_PARAMS", "FIXTURE_SHAPE", "bits_per",
    "ceil_log2", "delta", "human_bytes",
]
