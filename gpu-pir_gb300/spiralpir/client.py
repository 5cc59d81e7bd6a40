"""Spiral client: key generation, query encryption and response decoding.

The client is host-side and not part of the GPU answer path; the server
library only ever sees its public keys, its query ciphertext and the
response it returns.  It reproduces the conventions of the spiral-rs client
that generated the reference's golden vectors:

* Regev ciphertexts are [-a; s*a + e + m] (row 0, row 1); S = [s, 1].
* Expansion keys W_r (2 x t_exp) encrypt tau_{D/2^r+1}(s) * g^T; the
  server's coefficient expansion (gpu-pir/expansion.cuh:87-166) switches
  tau(s) back to s with them.
* The conversion key V (2 x 2*t_conv) encrypts s^2 * 2^(b k) in column 2k and
  s * 2^(b k) in column 2k+1, so V * G^-1(c) decrypts to s * (s c0 + c1).
* Packing keys W_r (n+1 x t_conv) encrypt, under the matrix secret
  S~ = [s~ | I_n], the vector with s * 2^(b k) in row r.
* Query polynomial: coefficient 2*row = Delta / 2^g; coefficient
  2*(i*t_gsw + j) + 1 = bit_i(col) * 2^(b_gsw j) / 2^(stop+1).

All key/ciphertext arrays are returned uint32 in the layouts of the C ABI
(rows, cols, 2, D) before conversion to u64 (`as_u64`).
"""
from __future__ import annotations

import dataclasses

import numpy as np

from . import prg, ring
from .params import D, Q, Q1, Q2, DbShape, SpiralParams, bits_per, delta

SIGMA = 6.4


def _gaussian(rng: np.random.Generator, shape) -> np.ndarray:
    """Rounded Gaussian with standard deviation 6.4 (int64)."""
    return np.rint(rng.normal(0.0, SIGMA, size=shape)).astype(np.int64)


def _uniform_ntt(rng: np.random.Generator, shape) -> np.ndarray:
    out = np.empty(tuple(shape) + (2, D), dtype=np.uint64)
    out[..., 0, :] = rng.integers(0, Q1, size=tuple(shape) + (D,), dtype=np.uint64)
    out[..., 1, :] = rng.integers(0, Q2, size=tuple(shape) + (D,), dtype=np.uint64)
    return out


def as_u64(a: np.ndarray) -> np.ndarray:
    """Residue arrays in the spiral-rs u64 CRT form used at the C ABI."""
    return np.ascontiguousarray(a, dtype=np.uint64)


@dataclasses.dataclass
class PublicKeys:
    exp_left: np.ndarray    # uint32 (n_left, 2, t_exp_left, 2, D)
    exp_right: np.ndarray   # uint32 (n_right, 2, t_exp_right, 2, D)
    conv: np.ndarray        # uint32 (2, 2*t_conv, 2, D)
    pack: np.ndarray        # uint32 (n, n+1, t_conv, 2, D)

    def nbytes_u64(self) -> int:
        return 2 * (self.exp_left.nbytes + self.exp_right.nbytes + self.conv.nbytes + self.pack.nbytes)


class Client:
    """One Spiral client with a seeded secret."""

    def __init__(self, params: SpiralParams, seed: int = 0):
        self.params = params
        self.rng = np.random.default_rng(seed)
        self.s = _gaussian(self.rng, (D,))                  # Regev secret
        self.s_gsw = _gaussian(self.rng, (params.n, D))     # matrix secret s~
        self.s_ntt = ring.to_ntt(ring.signed_to_raw(self.s))
        self.s_gsw_ntt = ring.to_ntt(ring.signed_to_raw(self.s_gsw))

    # -- encryption ------------------------------------------------------
    def _uniform_rows(self, lead) -> np.ndarray:
        """Uniform NTT polynomials for row 0 of the next key ciphertexts: the
        seeded stream (prg.seeded_poly, in key-set order) while a seeded key
        set is being made, else the negation of the client's generator draw."""
        if getattr(self, "_seed", None) is None:
            return ring.neg(_uniform_ntt(self.rng, lead))
        n = int(np.prod(lead, dtype=np.int64)) if lead else 1
        out = np.stack([prg.seeded_poly(self._seed, self._seed_next + i) for i in range(n)])
        self._seed_next += n
        return out.reshape(tuple(lead) + (2, D))

    def _enc(self, m_ntt: np.ndarray) -> np.ndarray:
        """Regev encryption of NTT-form messages (..., 2, D) -> (..., 2 rows, 2, D)."""
        m_ntt = np.asarray(m_ntt, dtype=np.uint64)
        lead = m_ntt.shape[:-2]
        a = ring.neg(self._uniform_rows(lead))      # row 0 = -a is the uniform row
        e = ring.to_ntt(ring.signed_to_raw(_gaussian(self.rng, lead + (D,))))
        b = ring.add(ring.add(ring.mul(self.s_ntt, a), e), m_ntt)
        return np.stack((ring.neg(a), b), axis=-3)

    def _gadget_cols(self, t: int) -> list[int]:
        b = bits_per(t)
        return [(1 << (b * k)) % Q if b * k < 64 else 0 for k in range(t)]

    def expansion_keys(self, count: int, t_exp: int) -> np.ndarray:
        """(count, 2, t_exp, 2, D): W_r = Enc_s(tau_{D/2^r+1}(s) * g^T)."""
        out = np.empty((count, 2, t_exp, 2, D), dtype=np.uint64)
        g = self._gadget_cols(t_exp)
        s_raw = ring.signed_to_raw(self.s)
        for r in range(count):
            tau_s = ring.to_ntt(ring.automorph(s_raw, (D >> r) + 1))
            msgs = np.stack([ring.mul(tau_s, ring.const_ntt(gk)) for gk in g])
            ct = self._enc(msgs)                     # (t_exp, 2 rows, 2, D)
            out[r] = np.transpose(ct, (1, 0, 2, 3))
        return out.astype(np.uint32)

    def conversion_key(self) -> np.ndarray:
        t = self.params.t_conv
        g = self._gadget_cols(t)
        s2 = ring.mul(self.s_ntt, self.s_ntt)
        msgs = []
        for k in range(t):
            msgs.append(ring.mul(s2, ring.const_ntt(g[k])))
            msgs.append(ring.mul(self.s_ntt, ring.const_ntt(g[k])))
        ct = self._enc(np.stack(msgs))                # (2t, 2 rows, 2, D)
        return np.transpose(ct, (1, 0, 2, 3)).astype(np.uint32)

    def packing_keys(self) -> np.ndarray:
        n, t = self.params.n, self.params.t_conv
        g = self._gadget_cols(t)
        out = np.empty((n, n + 1, t, 2, D), dtype=np.uint64)
        for r in range(n):
            for k in range(t):
                a = ring.neg(self._uniform_rows(()))
                out[r, 0, k] = ring.neg(a)
                for i in range(n):
                    e = ring.to_ntt(ring.signed_to_raw(_gaussian(self.rng, (D,))))
                    v = ring.add(ring.mul(self.s_gsw_ntt[i], a), e)
                    if i == r:
                        v = ring.add(v, ring.mul(self.s_ntt, ring.const_ntt(g[k])))
                    out[r, 1 + i, k] = v
        return out.astype(np.uint32)

    def public_keys(self, max_nu1: int, max_nu2: int, seed: bytes | None = None) -> PublicKeys:
        """Keys for any database with nu1 <= max_nu1 and nu2 <= max_nu2.
        With a 32-byte `seed`, row 0 of every key matrix is the seeded stream
        (prg.seeded_poly), so the server can regenerate it
        (SpiralGPU.set_client_keys_seeded); the keys are returned in full."""
        p = self.params
        g = max(p.g(a, b) for a in range(1, max_nu1 + 1) for b in range(1, max_nu2 + 1))
        stop = max(p.stop_round(b) for b in range(1, max_nu2 + 1))
        if seed is not None and len(bytes(seed)) != 32:
            raise ValueError("the seed is 32 bytes")
        self._seed, self._seed_next = (bytes(seed), 0) if seed is not None else (None, 0)
        try:
            return PublicKeys(
                exp_left=self.expansion_keys(g, p.t_exp_left),
                exp_right=self.expansion_keys(stop + 1, p.t_exp_right),
                conv=self.conversion_key(),
                pack=self.packing_keys(),
            )
        finally:
            self._seed = None

    # -- query -------------------------------------------------------------
    def query_poly(self, shape: DbShape, index: int) -> np.ndarray:
        """Raw query polynomial sigma (uint64 (D,) mod q) for record `index`."""
        p = self.params
        row, col = divmod(int(index), shape.cols)
        if not (0 <= row < shape.rows):
            raise IndexError("record index out of range")
        g = p.g(shape.nu1, shape.nu2)
        if 2 * p.t_gsw * shape.nu2 > (1 << g):
            raise ValueError("2^nu1 must be at least t_gsw*nu2 for the expansion layout")
        rest = min(p.stop_round(shape.nu2) + 1, g)
        sigma = np.zeros(D, dtype=object)
        sigma[2 * row] = delta(p) * pow(1 << g, -1, Q) % Q
        b = bits_per(p.t_gsw)
        inv_rest = pow(1 << rest, -1, Q)
        for i in range(shape.nu2):
            bit = (col >> i) & 1
            for j in range(p.t_gsw):
                sigma[2 * (i * p.t_gsw + j) + 1] = (bit << (b * j)) % Q * inv_rest % Q
        return np.array([int(x) for x in sigma], dtype=np.uint64)

    def query(self, shape: DbShape, index: int) -> np.ndarray:
        """Query ciphertext, uint32 (2 rows, 2, D) NTT form."""
        return self._enc(ring.to_ntt(self.query_poly(shape, index))).astype(np.uint32)

    # -- decoding ----------------------------------------------------------
    def decode(self, response: np.ndarray) -> np.ndarray:
        """Response bytes -> record plaintext uint8 (n*n, D)."""
        p = self.params
        n, q2, q1 = p.n, 1 << p.q2_bits, 1 << (p.pt_bits + 2)
        bits = np.unpackbits(np.asarray(response, dtype=np.uint8), bitorder="little")
        first_cnt, rest_cnt = n * D, n * n * D
        b0 = bits[: first_cnt * p.q2_bits].reshape(first_cnt, p.q2_bits).astype(np.int64)
        first = (b0 << np.arange(p.q2_bits, dtype=np.int64)).sum(axis=1).reshape(n, D)
        q1b = p.pt_bits + 2
        off = first_cnt * p.q2_bits
        b1 = bits[off: off + rest_cnt * q1b].reshape(rest_cnt, q1b).astype(np.int64)
        rest = (b1 << np.arange(q1b, dtype=np.int64)).sum(axis=1).reshape(n, n, D)
        out = np.empty((n * n, D), dtype=np.uint8)
        for r in range(n):
            for c in range(n):
                prod = ring.negacyclic_mul_small(self.s_gsw[r], first[c], q2)
                v = (ring.rescale_small(prod, q2, q1) + rest[r, c]) % q1
                out[r * n + c] = ring.rescale_small(v, q1, p.p).astype(np.uint8)
        return out

    def decode_margin(self, response: np.ndarray, expected: np.ndarray) -> float:
        """Largest distance, in units of the rows' modulus 4p, between the
        value decoded before the final rounding and its expected plaintext
        multiple (decoding fails at 2.0)."""
        p = self.params
        n, q2, q1 = p.n, 1 << p.q2_bits, 1 << (p.pt_bits + 2)
        bits = np.unpackbits(np.asarray(response, dtype=np.uint8), bitorder="little")
        first_cnt, rest_cnt = n * D, n * n * D
        b0 = bits[: first_cnt * p.q2_bits].reshape(first_cnt, p.q2_bits).astype(np.int64)
        first = (b0 << np.arange(p.q2_bits, dtype=np.int64)).sum(axis=1).reshape(n, D)
        q1b = p.pt_bits + 2
        off = first_cnt * p.q2_bits
        b1 = bits[off: off + rest_cnt * q1b].reshape(rest_cnt, q1b).astype(np.int64)
        rest = (b1 << np.arange(q1b, dtype=np.int64)).sum(axis=1).reshape(n, n, D)
        worst = 0.0
        for r in range(n):
            for c in range(n):
                prod = ring.negacyclic_mul_small(self.s_gsw[r], first[c], q2)
                exact = prod.astype(np.float64) * q1 / q2            # unrounded rescale
                v = (exact + rest[r, c]) % q1
                m = expected[r * n + c].astype(np.float64) * (q1 // p.p)
                d = np.abs(((v - m + q1 / 2) % q1) - q1 / 2)
                worst = max(worst, float(d.max()))
        return worst

    def decode_noise(self, packed_raw: np.ndarray, expected: np.ndarray) -> float:
        """log2 of the largest |noise| of a packed (n+1) x n raw ciphertext
        before modulus switching, against the expected record (diagnostic)."""
        p = self.params
        n = p.n
        worst = 0
        dl = delta(p)
        for r in range(n):
            for c in range(n):
                acc = np.zeros(D, dtype=object)
                s = [int(x) for x in self.s_gsw[r]]
                a = [int(x) for x in packed_raw[0, c]]
                full = np.convolve(np.array(s, dtype=object), np.array(a, dtype=object))
                acc[:] = full[:D]
                acc[: D - 1] -= full[D:]
                v = (acc + np.array([int(x) for x in packed_raw[1 + r, c]], dtype=object)) % Q
                m = np.array([int(x) for x in expected[r * n + c]], dtype=object)
                m = np.where(m > p.p // 2, m - p.p, m)
                e = (v - dl * m) % Q
                e = np.where(e > Q // 2, e - Q, e)
                worst = max(worst, int(np.max(np.abs(e))))
        return float(np.log2(max(worst, 1)))


def random_records(shape: DbShape, params: SpiralParams, seed: int = 0) -> np.ndarray:
    """Seeded uniform plaintext records, uint8 (num_records, n*n, D)."""
    rng = np.random.default_rng(seed)
    return rng.integers(0, params.p, size=(shape.num_records, params.T, D), dtype=np.uint8)
