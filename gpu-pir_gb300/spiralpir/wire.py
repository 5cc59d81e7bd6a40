"""Wire format of the messages between a Spiral client and this server.

The payloads use the polynomial layouts of the reference's golden vectors
(written by spiral-rs): a CRT polynomial is D residues mod q1 then D mod q2,
a ciphertext is its rows one after the other, a key matrix is row-major.
Residues are below 2^28, so they travel as little-endian uint32 (the C ABI
takes them widened to uint64).  Every message starts with a 16-byte header:

    magic   4 bytes   b"SPQ1" query, b"SPK1" public parameters,
                      b"SPS1" seeded public parameters, b"SPR1" response
    n, pt_bits, t_exp_left, t_exp_right, t_gsw, t_conv, q2_bits  7 x uint8
    a       uint8     query: nu1; keys: n_left; response: 0
    b       uint8     query: nu2; keys: n_right; response: 0
    pad     3 bytes   zero

Messages:
* query   header + ciphertext uint32 [2 rows][2][D]                    (32 KiB)
* keys    header + left [n_left][2][t_left][2][D] + right [n_right][2][t_right][2][D]
          + conv [2][2 t_conv][2][D] + pack [n][n+1][t_conv][2][D], uint32
* seeded  header + 32-byte seed + the same matrices without row 0 (row 0
          of every matrix is regenerated from the seed, spiralpir/prg.py):
          left [n_left][t_left][2][D], right [n_right][t_right][2][D],
          conv [2 t_conv][2][D], pack [n][n][t_conv][2][D]
* response header + the response bytes (sp_response_bytes of the
          parameters: row 0 at q2_bits, rows 1..n at pt_bits + 2 bits per
          coefficient, least significant bit first)

Parsing checks the magic, the parameters against the expected ones and the
length, and raises ValueError otherwise.
"""
from __future__ import annotations

import struct

import numpy as np

from .client import PublicKeys
from .params import D, SpiralParams

_HDR = struct.Struct("<4s7BBB3x")


def _header(magic: bytes, p: SpiralParams, a: int = 0, b: int = 0) -> bytes:
    return _HDR.pack(magic, p.n, p.pt_bits, p.t_exp_left, p.t_exp_right, p.t_gsw, p.t_conv, p.q2_bits, a, b)


def _check_header(buf: bytes, magic: bytes, p: SpiralParams) -> tuple[int, int]:
    if len(buf) < _HDR.size:
        raise ValueError("message shorter than its header")
    m, n, pt, tl, tr, tg, tc, q2, a, b = _HDR.unpack_from(buf)
    if m != magic:
        raise ValueError(f"expected a {magic!r} message, got {m!r}")
    if (n, pt, tl, tr, tg, tc, q2) != (p.n, p.pt_bits, p.t_exp_left, p.t_exp_right, p.t_gsw, p.t_conv, p.q2_bits):
        raise ValueError("message parameters differ from the server's")
    return a, b


def _u32(a: np.ndarray) -> bytes:
    a = np.asarray(a)
    if a.size and int(a.max()) >= 1 << 32:
        raise ValueError("residues must be below 2^32")
    return np.ascontiguousarray(a, dtype="<u4").tobytes()


def _take(buf: bytes, off: int, shape: tuple) -> tuple[np.ndarray, int]:
    n = int(np.prod(shape)) * 4
    if off + n > len(buf):
        raise ValueError("message too short")
    return np.frombuffer(buf, dtype="<u4", count=n // 4, offset=off).reshape(shape).astype(np.uint32), off + n


def encode_query(p: SpiralParams, nu1: int, nu2: int, ct: np.ndarray) -> bytes:
    return _header(b"SPQ1", p, nu1, nu2) + _u32(np.reshape(ct, (2, 2, D)))


def decode_query(p: SpiralParams, buf: bytes) -> tuple[int, int, np.ndarray]:
    nu1, nu2 = _check_header(buf, b"SPQ1", p)
    ct, off = _take(buf, _HDR.size, (2, 2, D))
    if off != len(buf):
        raise ValueError("trailing bytes after the query")
    return nu1, nu2, ct


def _shapes(p: SpiralParams, n_left: int, n_right: int, seeded: bool) -> list[tuple]:
    rows = 1 if seeded else 2
    return [(n_left, rows, p.t_exp_left, 2, D), (n_right, rows, p.t_exp_right, 2, D),
            (rows, 2 * p.t_conv, 2, D), (p.n, p.n + 1 - (1 if seeded else 0), p.t_conv, 2, D)]


def encode_keys(p: SpiralParams, keys: PublicKeys) -> bytes:
    nl, nr = keys.exp_left.shape[0], keys.exp_right.shape[0]
    return _header(b"SPK1", p, nl, nr) + b"".join(_u32(x) for x in (keys.exp_left, keys.exp_right, keys.conv,
                                                                     keys.pack))


def decode_keys(p: SpiralParams, buf: bytes) -> PublicKeys:
    nl, nr = _check_header(buf, b"SPK1", p)
    off, parts = _HDR.size, []
    for shape in _shapes(p, nl, nr, False):
        a, off = _take(buf, off, shape)
        parts.append(a)
    if off != len(buf):
        raise ValueError("trailing bytes after the keys")
    return PublicKeys(*parts)


def encode_seeded_keys(p: SpiralParams, seed: bytes, keys: PublicKeys) -> bytes:
    """Keys made with Client.public_keys(..., seed=seed): only the rows
    below row 0 travel, with the seed."""
    if len(seed) != 32:
        raise ValueError("the seed is 32 bytes")
    nl, nr = keys.exp_left.shape[0], keys.exp_right.shape[0]
    rest = (keys.exp_left[:, 1:], keys.exp_right[:, 1:], keys.conv[1:], keys.pack[:, 1:])
    return _header(b"SPS1", p, nl, nr) + bytes(seed) + b"".join(_u32(x) for x in rest)


def decode_seeded_keys(p: SpiralParams, buf: bytes) -> tuple[bytes, PublicKeys]:
    """Returns the seed and PublicKeys whose row 0 planes are zero (the
    library regenerates them: SpiralGPU.set_client_keys_seeded)."""
    nl, nr = _check_header(buf, b"SPS1", p)
    if len(buf) < _HDR.size + 32:
        raise ValueError("message too short")
    seed = bytes(buf[_HDR.size:_HDR.size + 32])
    off, parts = _HDR.size + 32, []
    for shape in _shapes(p, nl, nr, True):
        a, off = _take(buf, off, shape)
        parts.append(a)
    if off != len(buf):
        raise ValueError("trailing bytes after the keys")
    left = np.zeros((nl, 2, p.t_exp_left, 2, D), np.uint32)
    left[:, 1:] = parts[0]
    right = np.zeros((nr, 2, p.t_exp_right, 2, D), np.uint32)
    right[:, 1:] = parts[1]
    conv = np.zeros((2, 2 * p.t_conv, 2, D), np.uint32)
    conv[1:] = parts[2]
    pack = np.zeros((p.n, p.n + 1, p.t_conv, 2, D), np.uint32)
    pack[:, 1:] = parts[3]
    return seed, PublicKeys(left, right, conv, pack)


def encode_response(p: SpiralParams, resp: np.ndarray) -> bytes:
    resp = np.asarray(resp, dtype=np.uint8)
    if resp.size != p.response_bytes():
        raise ValueError("response length differs from the parameters'")
    return _header(b"SPR1", p) + resp.tobytes()


def decode_response(p: SpiralParams, buf: bytes) -> np.ndarray:
    _check_header(buf, b"SPR1", p)
    body = np.frombuffer(buf, dtype=np.uint8, offset=_HDR.size)
    if body.size != p.response_bytes():
        raise ValueError("response length differs from the parameters'")
    return body.copy()


__all__ = ["encode_query", "decode_query", "encode_keys", "decode_keys", "encode_seeded_keys",
           "decode_seeded_keys", "encode_response", "decode_response"]
