"""Seed expansion of public parameters (host side).

The uniform rows of a client's key ciphertexts (row 0 of every expansion,
conversion and packing key matrix) carry no secret: the client can send a
32-byte seed instead and the server regenerates them (the plan of
gpu-pir/optplan.md:88-92).  The stream is the ChaCha20 block function of
RFC 8439 (20 rounds, 32-byte key, 32-bit block counter, 96-bit nonce),
restated here with numpy and in the library (csrc/seeded.cu):

* key   = the seed (eight little-endian 32-bit words);
* nonce = (poly index P, prime index k, SEED_DOMAIN), where P numbers the
  row-0 polynomials of a key set in the order: expansion-left matrices
  (matrix r, column j), expansion-right, conversion (column j), packing
  (matrix r, column j);
* block b (counter) gives residues z = 8b .. 8b+7: residue z is the 64-bit
  little-endian word of block words 2(z mod 8), 2(z mod 8)+1, reduced mod
  q_k (bias below 2^-35).

The residues are the row-0 polynomial itself in NTT form (spiral order).
"""
from __future__ import annotations

import numpy as np

from .params import D, Q1, Q2

SEED_DOMAIN = 0x3153504B          # "KPS1" little-endian: key-seed stream, version 1
_CONST = np.array([0x61707865, 0x3320646E, 0x79622D32, 0x6B206574], dtype=np.uint32)


def _rotl(x: np.ndarray, n: int) -> np.ndarray:
    return (x << np.uint32(n)) | (x >> np.uint32(32 - n))


def chacha20_blocks(key_words: np.ndarray, counters: np.ndarray, nonces: np.ndarray) -> np.ndarray:
    """ChaCha20 block function (RFC 8439 2.3) for many blocks at once.

    key_words uint32 (8,); counters uint32 (n,); nonces uint32 (n, 3).
    Returns the 16 output words of each block, uint32 (n, 16)."""
    n = counters.shape[0]
    st = np.empty((16, n), dtype=np.uint32)
    st[0:4] = _CONST[:, None]
    st[4:12] = np.asarray(key_words, dtype=np.uint32)[:, None]
    st[12] = counters
    st[13:16] = np.asarray(nonces, dtype=np.uint32).T
    x = st.copy()

    def qr(a, b, c, d):
        x[a] += x[b]; x[d] ^= x[a]; x[d] = _rotl(x[d], 16)
        x[c] += x[d]; x[b] ^= x[c]; x[b] = _rotl(x[b], 12)
        x[a] += x[b]; x[d] ^= x[a]; x[d] = _rotl(x[d], 8)
        x[c] += x[d]; x[b] ^= x[c]; x[b] = _rotl(x[b], 7)

    with np.errstate(over="ignore"):
        for _ in range(10):
            qr(0, 4, 8, 12); qr(1, 5, 9, 13); qr(2, 6, 10, 14); qr(3, 7, 11, 15)
            qr(0, 5, 10, 15); qr(1, 6, 11, 12); qr(2, 7, 8, 13); qr(3, 4, 9, 14)
        x += st
    return x.T.copy()


def seed_words(seed: bytes) -> np.ndarray:
    if len(seed) != 32:
        raise ValueError("the seed is 32 bytes")
    return np.frombuffer(seed, dtype="<u4").astype(np.uint32)


def seeded_poly(seed: bytes, index: int) -> np.ndarray:
    """Row-0 polynomial number `index` of the key set: uint64 (2, D) residues
    mod q1 and q2, NTT form."""
    kw = seed_words(seed)
    out = np.empty((2, D), dtype=np.uint64)
    blocks = np.arange(D // 8, dtype=np.uint32)
    for k, q in enumerate((Q1, Q2)):
        nonces = np.empty((blocks.size, 3), dtype=np.uint32)
        nonces[:, 0] = index
        nonces[:, 1] = k
        nonces[:, 2] = SEED_DOMAIN
        w = chacha20_blocks(kw, blocks, nonces).astype(np.uint64)     # (256, 16)
        v = w[:, 0::2] | (w[:, 1::2] << np.uint64(32))                 # (256, 8)
        out[k] = (v % np.uint64(q)).reshape(D)
    return out


__all__ = ["SEED_DOMAIN", "chacha20_blocks", "seed_words", "seeded_poly"]
