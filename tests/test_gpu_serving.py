"""GPU tests of batching and the serving loop: every result is the same
alone and in the mix (bit-exact), for both multiply variants, for queries
submitted concurrently from several threads against databases of different
shapes, and requests that cannot run complete with their error."""
import threading

import numpy as np
import pytest

from spiralpir import client as C
from spiralpir import params as P
from spiralpir.lib import SpiralError, SpiralGPU
from spiralpir.serving import Server, poisson_load

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def world():
    p = P.PARAMS
    gpu = SpiralGPU(p, max_batch=8)
    a, b = P.SHAPE_8MIB, P.DbShape(6, 4)
    ra = C.random_records(a, p, seed=61)
    rb = C.random_records(b, p, seed=62)
    gpu.load_db(1, ra, a.nu1, a.nu2)
    gpu.load_db(2, rb, b.nu1, b.nu2)
    clients = {}
    for cid in (1, 2, 3):
        cl = C.Client(p, seed=70 + cid)
        gpu.set_client_keys(cid, cl.public_keys(7, 4))
        clients[cid] = cl
    rng = np.random.default_rng(5)
    reqs = []
    for k in range(24):
        cid = 1 + k % 3
        did, sh, recs = (1, a, ra) if k % 2 == 0 else (2, b, rb)
        idx = int(rng.integers(0, sh.num_records))
        reqs.append((cid, did, clients[cid].query(sh, idx), idx, recs))
    alone = [gpu.answer(c, d, q) for c, d, q, _, _ in reqs]
    yield gpu, clients, reqs, alone
    gpu.close()


def test_alone_results_decode(world):
    gpu, clients, reqs, alone = world
    for (cid, _, _, idx, recs), r in zip(reqs, alone):
        assert np.array_equal(clients[cid].decode(r), recs[idx])


@pytest.mark.parametrize("variant", [1, 2, 0])
def test_batch_variants_match_alone(world, variant):
    gpu, _, reqs, alone = world
    gpu.set_db_mul_variant(variant)
    try:
        for s in range(0, len(reqs), 8):
            got = gpu.answer_batch([(c, d, q) for c, d, q, _, _ in reqs[s:s + 8]])
            for x, y in zip(got, alone[s:s + 8]):
                assert np.array_equal(x, y)
    finally:
        gpu.set_db_mul_variant(0)


def test_serving_threads_match_alone(world):
    gpu, _, reqs, alone = world
    out = [None] * len(reqs)
    with Server(gpu, lanes=2) as srv:
        def worker(ks):
            ts = [(k, srv.submit(reqs[k][0], reqs[k][1], reqs[k][2])) for k in ks]
            for k, t in ts:
                out[k] = t.result().copy()
        th = [threading.Thread(target=worker, args=(list(range(i, len(reqs), 4)),)) for i in range(4)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        st = srv.stats()
    assert st["served"] == len(reqs)
    for x, y in zip(out, alone):
        assert np.array_equal(x, y)


def test_serving_poisson_and_errors(world):
    gpu, _, reqs, alone = world
    with Server(gpu, lanes=2) as srv:
        res = poisson_load(srv, [(c, d, q) for c, d, q, _, _ in reqs], rate_qps=2000.0, seed=3)
        bad = srv.submit(99, 1, reqs[0][2])
        with pytest.raises(SpiralError) as e:
            bad.result()
        assert e.value.code == 4
    for x, y in zip(res["responses"], alone):
        assert np.array_equal(x, y)
    assert res["p99_ms"] >= res["p50_ms"] > 0
