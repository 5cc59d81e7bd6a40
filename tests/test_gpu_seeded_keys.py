"""Seed-compressed public parameters: a client sends a 32-byte seed in place
of row 0 of every key matrix, and the library regenerates those rows on the
device (ChaCha20 stream, csrc/seeded.cu).  Answers with keys registered this
way are byte-identical to answers with the same keys sent in full, and
decode to the records."""
import numpy as np
import pytest

from spiralpir import client as C
from spiralpir import params as P
from spiralpir import wire
from spiralpir.lib import SpiralGPU

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("params, shape", [(P.PARAMS, P.SHAPE_8MIB), (P.FIXTURE_PARAMS, P.FIXTURE_SHAPE)])
def test_seeded_keys_give_the_same_answers(params, shape):
    seed = bytes(range(3, 35))
    cl = C.Client(params, seed=71)
    keys = cl.public_keys(shape.nu1, shape.nu2, seed=seed)
    recs = C.random_records(shape, params, seed=72)
    with SpiralGPU(params, max_batch=4) as gpu:
        gpu.set_client_keys(1, keys)
        gpu.set_client_keys_seeded(2, seed, keys)
        gpu.load_db(1, recs, shape.nu1, shape.nu2)
        idx = [0, shape.num_records - 1, 77]
        qs = [cl.query(shape, i) for i in idx]
        for i, q in zip(idx, qs):
            full = gpu.answer(1, 1, q)
            seeded = gpu.answer(2, 1, q)
            assert np.array_equal(full, seeded)
            assert np.array_equal(cl.decode(seeded), recs[i])
        batch = gpu.answer_batch([(2, 1, q) for q in qs])
        for i, r in zip(idx, batch):
            assert np.array_equal(cl.decode(r), recs[i])


def test_seeded_keys_with_a_wrong_seed_do_not_decode():
    seed = bytes(range(32))
    p, sh = P.PARAMS, P.SHAPE_8MIB
    cl = C.Client(p, seed=73)
    keys = cl.public_keys(sh.nu1, sh.nu2, seed=seed)
    recs = C.random_records(sh, p, seed=74)
    with SpiralGPU(p) as gpu:
        gpu.set_client_keys_seeded(1, bytes(32), keys)       # not the client's seed
        gpu.load_db(1, recs, sh.nu1, sh.nu2)
        r = gpu.answer(1, 1, cl.query(sh, 5))
        assert not np.array_equal(cl.decode(r), recs[5])
        with pytest.raises(ValueError):
            gpu.set_client_keys_seeded(2, b"short", keys)


def test_seeded_keys_over_the_wire():
    """Client -> server messages (seeded keys, query) and the response back,
    through the wire format; the record decodes."""
    p, sh = P.PARAMS, P.SHAPE_8MIB
    seed = bytes(range(100, 132))
    cl = C.Client(p, seed=75)
    recs = C.random_records(sh, p, seed=76)
    key_msg = wire.encode_seeded_keys(p, seed, cl.public_keys(sh.nu1, sh.nu2, seed=seed))
    query_msg = wire.encode_query(p, sh.nu1, sh.nu2, cl.query(sh, 321))
    with SpiralGPU(p) as gpu:
        gpu.load_db(1, recs, sh.nu1, sh.nu2)
        s, keys = wire.decode_seeded_keys(p, key_msg)
        gpu.set_client_keys_seeded(9, s, keys)
        _, _, q = wire.decode_query(p, query_msg)
        resp_msg = wire.encode_response(p, gpu.answer(9, 1, q))
    assert np.array_equal(cl.decode(wire.decode_response(p, resp_msg)), recs[321])
