"""Wire format (spiralpir/wire.py): queries, public parameters (full and
seeded) and responses survive a round trip byte for byte; headers and
lengths are checked; the seeded form carries a quarter of the full keys'
uint64 bytes."""
import numpy as np
import pytest

from spiralpir import client as C
from spiralpir import params as P
from spiralpir import wire


@pytest.fixture(scope="module")
def parts():
    p, sh = P.PARAMS, P.DbShape(6, 2)
    cl = C.Client(p, seed=31)
    seed = bytes(range(40, 72))
    return p, sh, cl, seed, cl.public_keys(sh.nu1, sh.nu2, seed=seed)


def test_query_round_trip(parts):
    p, sh, cl, _, _ = parts
    q = cl.query(sh, 9)
    buf = wire.encode_query(p, sh.nu1, sh.nu2, q)
    assert len(buf) == 16 + 2 * 2 * P.D * 4
    nu1, nu2, q2 = wire.decode_query(p, buf)
    assert (nu1, nu2) == (sh.nu1, sh.nu2) and np.array_equal(q2, q)


def test_keys_round_trip_full_and_seeded(parts):
    p, _, _, seed, keys = parts
    full = wire.encode_keys(p, keys)
    k2 = wire.decode_keys(p, full)
    for f in ("exp_left", "exp_right", "conv", "pack"):
        assert np.array_equal(getattr(k2, f), getattr(keys, f))
    sb = wire.encode_seeded_keys(p, seed, keys)
    s2, k3 = wire.decode_seeded_keys(p, sb)
    assert s2 == seed
    assert np.array_equal(k3.exp_left[:, 1], keys.exp_left[:, 1]) and not k3.exp_left[:, 0].any()
    assert np.array_equal(k3.pack[:, 1:], keys.pack[:, 1:]) and not k3.pack[:, 0].any()
    # uint32 payloads, and about half the rows: well under a quarter of the
    # uint64 form the C ABI takes
    assert len(sb) < 0.3 * keys.nbytes_u64()


def test_response_round_trip_and_checks(parts):
    p, _, _, _, _ = parts
    resp = np.arange(p.response_bytes(), dtype=np.uint64).astype(np.uint8)
    buf = wire.encode_response(p, resp)
    assert np.array_equal(wire.decode_response(p, buf), resp)
    with pytest.raises(ValueError):
        wire.decode_response(p, buf[:-1])
    with pytest.raises(ValueError):
        wire.decode_query(p, buf)                                   # wrong magic
    other = P.SpiralParams(n=1)
    with pytest.raises(ValueError):
        wire.decode_response(other, wire.encode_response(p, resp))  # parameters differ
