"""Host-side ring arithmetic for the Spiral client (numpy).

The client (key generation, query encryption, response decoding) runs on
the host and is not part of the server answer path.  It needs the same NTT
order as the server: the in-place Cooley-Tukey negacyclic transform with
bit-reversed powers of the primitive 4096-th root psi, the order spiral-rs
and the reference use (gpu-pir/host.cu:64-71, gpu-pir/ntt_28bit.cuh:31-131).

Arrays: NTT form uint64 (..., 2, D) (residues mod q1, q2); raw uint64
(..., D) mod q.
"""
from __future__ import annotations

import functools

import numpy as np

from .params import D, Q, Q1, Q2

PRIMES = (Q1, Q2)
_PSI = (66687, 158221)


def _brev(x: int, bits: int) -> int:
    r = 0
    for _ in range(bits):
        r = (r << 1) | (x & 1)
        x >>= 1
    return r


@functools.lru_cache(maxsize=None)
def _tables():
    fwd, inv, ninv = [], [], []
    for p, psi in zip(PRIMES, _PSI):
        psi_inv = pow(psi, 4095, p)
        b = [_brev(i, 11) for i in range(D)]
        fwd.append(np.array([pow(psi, e, p) for e in b], dtype=np.uint64))
        inv.append(np.array([pow(psi_inv, e, p) for e in b], dtype=np.uint64))
        ninv.append(pow(D, p - 2, p))
    return fwd, inv, ninv


def ntt(res: np.ndarray) -> np.ndarray:
    """Forward NTT of canonical residues uint64 (..., 2, D)."""
    fwd, _, _ = _tables()
    res = np.asarray(res, dtype=np.uint64)
    out = np.empty_like(res)
    lead = res.shape[:-2]
    for k, p in enumerate(PRIMES):
        x = res[..., k, :].reshape(-1, D).copy()
        pp = np.uint64(p)
        m, h = 1, D // 2
        while m < D:
            x = x.reshape(-1, m, 2, h)
            s = fwd[k][m:2 * m].reshape(1, m, 1)
            u = x[:, :, 0, :]
            v = (x[:, :, 1, :] * s) % pp
            x = np.stack(((u + v) % pp, (u + pp - v) % pp), axis=2)
            m, h = m * 2, h // 2
        out[..., k, :] = x.reshape(lead + (D,))
    return out


def intt(a: np.ndarray) -> np.ndarray:
    """Inverse NTT including the 2048^-1 scaling, uint64 (..., 2, D)."""
    _, inv, ninv = _tables()
    a = np.asarray(a, dtype=np.uint64)
    out = np.empty_like(a)
    lead = a.shape[:-2]
    for k, p in enumerate(PRIMES):
        x = a[..., k, :].reshape(-1, D).copy()
        pp = np.uint64(p)
        m, h = D // 2, 1
        while m >= 1:
            x = x.reshape(-1, m, 2, h)
            s = inv[k][m:2 * m].reshape(1, m, 1)
            u = x[:, :, 0, :]
            v = x[:, :, 1, :]
            x = np.stack(((u + v) % pp, ((u + pp - v) * s) % pp), axis=2)
            m, h = m // 2, h * 2
        out[..., k, :] = (x.reshape(lead + (D,)) * np.uint64(ninv[k])) % pp
    return out


def crt_split(raw: np.ndarray) -> np.ndarray:
    """raw uint64 (..., D) mod q -> residues uint64 (..., 2, D)."""
    raw = np.asarray(raw, dtype=np.uint64)
    return np.stack((raw % np.uint64(Q1), raw % np.uint64(Q2)), axis=-2)


_M1 = pow(Q2, Q1 - 2, Q1)
_M2 = pow(Q1, Q2 - 2, Q2)


def crt_join(res: np.ndarray) -> np.ndarray:
    """residues uint64 (..., 2, D) -> raw uint64 (..., D) mod q."""
    a = (res[..., 0, :].astype(np.uint64) * np.uint64(_M1)) % np.uint64(Q1)
    b = (res[..., 1, :].astype(np.uint64) * np.uint64(_M2)) % np.uint64(Q2)
    # a*q2 + b*q1 < 2q < 2^57: exact in uint64
    s = a * np.uint64(Q2) + b * np.uint64(Q1)
    return np.where(s >= np.uint64(Q), s - np.uint64(Q), s)


def to_ntt(raw: np.ndarray) -> np.ndarray:
    return ntt(crt_split(raw))


def from_ntt(a: np.ndarray) -> np.ndarray:
    return crt_join(intt(a))


def signed_to_raw(x: np.ndarray) -> np.ndarray:
    """int64 small signed coefficients -> uint64 mod q."""
    x = np.asarray(x, dtype=np.int64)
    return np.where(x < 0, (np.int64(Q) + x), x).astype(np.uint64)


def const_ntt(c: int, shape=()) -> np.ndarray:
    """NTT form of the constant polynomial c (c mod q): c mod q_i in every slot."""
    out = np.empty(tuple(shape) + (2, D), dtype=np.uint64)
    out[..., 0, :] = c % Q1
    out[..., 1, :] = c % Q2
    return out


def mul(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Pointwise product of NTT forms."""
    p = np.array(PRIMES, dtype=np.uint64).reshape(2, 1)
    return (np.asarray(a, dtype=np.uint64) * np.asarray(b, dtype=np.uint64)) % p


def add(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    p = np.array(PRIMES, dtype=np.uint64).reshape(2, 1)
    return (np.asarray(a, dtype=np.uint64) + np.asarray(b, dtype=np.uint64)) % p


def neg(a: np.ndarray) -> np.ndarray:
    p = np.array(PRIMES, dtype=np.uint64).reshape(2, 1)
    return (p - np.asarray(a, dtype=np.uint64)) % p


def automorph(raw: np.ndarray, t: int) -> np.ndarray:
    """x -> x^t on raw coefficients mod q (negacyclic)."""
    raw = np.asarray(raw, dtype=np.uint64)
    i = np.arange(D, dtype=np.int64)
    it = i * t
    idx = it % D
    flip = (it // D) % 2 == 1
    vals = np.where(flip, np.where(raw == 0, raw, np.uint64(Q) - raw), raw)
    out = np.empty_like(raw)
    out[..., idx] = vals
    return out


def negacyclic_mul_small(s: np.ndarray, a: np.ndarray, modulus: int) -> np.ndarray:
    """(s * a) mod (x^D + 1, modulus) for small signed int64 s and int64 a in
    [0, modulus); exact as long as |s|_1 * modulus < 2^63."""
    full = np.convolve(np.asarray(s, dtype=np.int64), np.asarray(a, dtype=np.int64))
    res = full[:D].copy()
    res[: D - 1] -= full[D:]
    return np.mod(res, modulus)


def rescale(x: np.ndarray, q_in: int, q_out: int) -> np.ndarray:
    """round(x * q_out / q_in) mod q_out for x in Z_{q_in} read as centred,
    ties away from zero (Python-int exact)."""
    x = np.asarray(x).astype(object) % q_in
    half = (q_in + 1) // 2
    out = np.empty(x.shape, dtype=np.int64)
    flat_in, flat_out = x.reshape(-1), out.reshape(-1)
    for i, v in enumerate(flat_in):
        v = int(v)
        if v >= half:
            y = ((q_in - v) * q_out + q_in // 2) // q_in % q_out
            flat_out[i] = (q_out - y) % q_out
        else:
            flat_out[i] = (v * q_out + q_in // 2) // q_in % q_out
    return out


def rescale_small(x: np.ndarray, q_in: int, q_out: int) -> np.ndarray:
    """rescale() for q_in * q_out < 2^62 (vectorised in int64)."""
    x = np.asarray(x, dtype=np.int64) % q_in
    half = (q_in + 1) // 2
    pos = (x * q_out + q_in // 2) // q_in % q_out
    negv = ((q_in - x) * q_out + q_in // 2) // q_in % q_out
    return np.where(x >= half, (q_out - negv) % q_out, pos)
