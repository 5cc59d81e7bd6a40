"""Byte-exact parity at the headline configuration: a 1 GiB database
(nu1 = 9, nu2 = 8, n = 2, p = 256: 2^17 records of 8 KiB, a 7 GiB image on
the device), d = 2048, t_exp = 8, t_gsw = 7, t_conv = 4.

* one query answered on the GPU gives exactly the oracle's response bytes
  (the oracle encodes the whole database on the host: 8 GiB of u32 planes);
* batches of 32 and 64 distinct queries from two clients give, slot for slot,
  the bytes of the same queries answered alone, and every response decodes to
  its record;
* the larger parameter set of gpu-pir/params.cuh:57-62 (t_exp_left = 16,
  t_exp_right = 56, nu1 = 10, nu2 = 4) equals the oracle byte for byte.
"""
import numpy as np
import pytest

import oracle as O
from spiralpir import client as C
from spiralpir import params as P
from spiralpir.lib import SpiralGPU

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def headline():
    p, sh = P.PARAMS, P.SHAPE_1GIB
    clients = [C.Client(p, seed=601), C.Client(p, seed=611)]
    keys = [cl.public_keys(sh.nu1, sh.nu2) for cl in clients]
    recs = C.random_records(sh, p, seed=602)
    gpu = SpiralGPU(p, max_batch=64)
    for k, ks in enumerate(keys):
        gpu.set_client_keys(1 + k, ks)
    gpu.load_db(1, recs, sh.nu1, sh.nu2)
    yield p, sh, clients, keys, recs, gpu
    gpu.close()


def _oracle_answer(db, q, keys, p, sh):
    return O.answer(db, q, keys.exp_left, keys.exp_right, keys.conv, keys.pack, n=p.n, nu1=sh.nu1, nu2=sh.nu2,
                    pt_bits=p.pt_bits, q2_bits=p.q2_bits, t_left=p.t_exp_left, t_right=p.t_exp_right,
                    t_gsw=p.t_gsw, t_conv=p.t_conv)


def test_1gib_answer_equals_oracle(headline):
    p, sh, clients, keys, recs, gpu = headline
    db = O.db_encode(recs, p.n, sh.nu1, sh.nu2, p.pt_bits)
    try:
        for k, idx in ((0, sh.num_records - 1), (1, 70001)):
            q = clients[k].query(sh, idx)
            resp = gpu.answer(1 + k, 1, q)
            ref = _oracle_answer(db, q, keys[k], p, sh)
            assert np.array_equal(resp, ref), f"client {k}, record {idx}"
            assert np.array_equal(clients[k].decode(resp), recs[idx])
    finally:
        del db


@pytest.mark.parametrize("B", [32, 64])
def test_1gib_batch_equals_single(headline, B):
    p, sh, clients, keys, recs, gpu = headline
    rng = np.random.default_rng(620 + B)
    idx = [int(x) for x in rng.choice(sh.num_records, size=B, replace=False)]
    reqs = [(1 + s % 2, 1, clients[s % 2].query(sh, i)) for s, i in enumerate(idx)]
    alone = [gpu.answer(c, d, q) for c, d, q in reqs]
    batch = gpu.answer_batch(reqs)
    for s, (x, y) in enumerate(zip(batch, alone)):
        assert np.array_equal(x, y), f"slot {s}"
        assert np.array_equal(clients[s % 2].decode(x), recs[idx[s]]), f"slot {s}"


def test_production_parameter_set_equals_oracle():
    p = P.SpiralParams(n=2, pt_bits=8, t_exp_left=16, t_exp_right=56, t_gsw=7, t_conv=4, q2_bits=22)
    sh = P.DbShape(10, 4)
    recs = C.random_records(sh, p, seed=121)
    cl = C.Client(p, seed=122)
    keys = cl.public_keys(sh.nu1, sh.nu2)
    db = O.db_encode(recs, p.n, sh.nu1, sh.nu2, p.pt_bits)
    with SpiralGPU(p, max_batch=2) as gpu:
        gpu.set_client_keys(1, keys)
        gpu.load_db(1, recs, sh.nu1, sh.nu2)
        for i in (3, sh.num_records - 2):
            q = cl.query(sh, i)
            resp = gpu.answer(1, 1, q)
            assert np.array_equal(resp, _oracle_answer(db, q, keys, p, sh)), f"record {i}"
            assert np.array_equal(cl.decode(resp), recs[i])
