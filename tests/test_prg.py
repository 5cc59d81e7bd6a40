"""Seed expansion of public parameters on the host (spiralpir/prg.py): the
ChaCha20 block function against known-answer vectors of an independent
implementation (tests/golden/chacha20.json, made by make_chacha_vectors.py),
and the seeded key rows of the client."""
import json
import os

import numpy as np

from spiralpir import client as C
from spiralpir import params as P
from spiralpir import prg

VECTORS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "chacha20.json")))


def test_chacha20_block_known_answers():
    assert VECTORS[0]["block"].startswith("10f1e7e4d13b5915")     # RFC 8439 section 2.3.2
    for v in VECTORS:
        key = bytes.fromhex(v["key"])
        nonce = np.frombuffer(bytes.fromhex(v["nonce"]), dtype="<u4")[None]
        got = prg.chacha20_blocks(prg.seed_words(key), np.array([v["counter"]], np.uint32), nonce)
        assert got.astype("<u4").tobytes().hex() == v["block"]


def test_seeded_poly_range_and_determinism():
    seed = bytes(range(32))
    a = prg.seeded_poly(seed, 3)
    assert a.shape == (2, P.D) and a[0].max() < P.Q1 and a[1].max() < P.Q2
    assert np.array_equal(a, prg.seeded_poly(seed, 3))
    assert not np.array_equal(a, prg.seeded_poly(seed, 4))
    assert not np.array_equal(a, prg.seeded_poly(bytes(32), 3))


def test_seeded_keys_place_the_stream_in_row0():
    """Row 0 of every key matrix is the seeded stream in key-set order:
    left (matrix, column), right, conversion, packing (matrix, column)."""
    p = P.PARAMS
    seed = bytes(range(7, 39))
    k = C.Client(p, seed=9).public_keys(6, 2, seed=seed)
    idx = 0
    for mats in (k.exp_left, k.exp_right):
        for r in range(mats.shape[0]):
            for j in range(mats.shape[2]):
                if j in (0, mats.shape[2] - 1):
                    assert np.array_equal(mats[r, 0, j].astype(np.uint64), prg.seeded_poly(seed, idx))
                idx += 1
    for j in range(2 * p.t_conv):
        if j in (0, 2 * p.t_conv - 1):
            assert np.array_equal(k.conv[0, j].astype(np.uint64), prg.seeded_poly(seed, idx))
        idx += 1
    for r in range(p.n):
        for j in range(p.t_conv):
            assert np.array_equal(k.pack[r, 0, j].astype(np.uint64), prg.seeded_poly(seed, idx))
            idx += 1


def test_unseeded_keys_unchanged_by_the_seeded_path():
    """Keys made without a seed depend only on the client seed (same draws
    as before the seeded path existed)."""
    p = P.PARAMS
    a = C.Client(p, seed=5).public_keys(6, 2)
    b = C.Client(p, seed=5).public_keys(6, 2)
    for f in ("exp_left", "exp_right", "conv", "pack"):
        assert np.array_equal(getattr(a, f), getattr(b, f))
