"""GPU tests of batching and the serving loop: every result is the same
alone and in the mix (bit-exact), for every multiply variant, for queries
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


def test_graph_replay_matches_direct_launches(world):
    """The same batch plan run with plain launches, then captured (second
    run) and replayed: every response is identical to the query alone."""
    gpu, _, reqs, alone = world
    batch = [(c, d, q) for c, d, q, _, _ in reqs[:8]]
    try:
        gpu.set_graphs(False)
        direct = gpu.answer_batch(batch)
        gpu.set_graphs(True)
        runs = [gpu.answer_batch(batch) for _ in range(3)]
    finally:
        gpu.set_graphs(True)
    for got in [direct] + runs:
        for x, y in zip(got, alone[:8]):
            assert np.array_equal(x, y)


@pytest.mark.parametrize("variant", [1, 2])
def test_stage_timing_on_and_off_match_alone(world, variant):
    """With stage timing on (events between the stages) and off (the stages
    as dependent launches, per-query multiply included), plain launches and
    graph replays give every response of the query alone; the stage fields
    of the stats fill only with the timing on."""
    gpu, _, reqs, alone = world
    batch = [(c, d, q) for c, d, q, _, _ in reqs[:8]]
    gpu.set_db_mul_variant(variant)
    try:
        for timing in (True, False):
            gpu.set_stage_timing(timing)
            gpu.stats_reset()
            for _ in range(3):   # plain launches, capture, replay
                got = gpu.answer_batch(batch)
                for x, y in zip(got, alone[:8]):
                    assert np.array_equal(x, y)
            st = gpu.stats()
            assert st["ms_total"] > 0
            stages = sum(st[k] for k in ("ms_expand", "ms_db_mul", "ms_fold", "ms_pack"))
            assert (stages > 0) == timing
    finally:
        gpu.set_stage_timing(False)
        gpu.set_db_mul_variant(0)


def test_graphs_dropped_when_database_reloaded():
    """A captured plan refers to the database image; reloading the database
    under the same id must not replay stale pointers."""
    p = P.PARAMS
    sh = P.SHAPE_8MIB
    cl = C.Client(p, seed=81)
    with SpiralGPU(p, max_batch=4) as gpu:
        gpu.set_client_keys(1, cl.public_keys(sh.nu1, sh.nu2))
        for seed in (82, 83):
            recs = C.random_records(sh, p, seed=seed)
            gpu.load_db(1, recs, sh.nu1, sh.nu2)
            idx = [3, 500, 1000, 7]
            qs = [(1, 1, cl.query(sh, i)) for i in idx]
            for _ in range(3):           # plain, captured, replayed
                for i, r in zip(idx, gpu.answer_batch(qs)):
                    assert np.array_equal(cl.decode(r), recs[i])


def test_graphs_dropped_when_slots_grow():
    """Captured plans copy queries and responses through the lane's slot
    buffers; a query to a larger database reallocates every slot, after
    which the small database's plan must be captured again, not replayed."""
    p = P.PARAMS
    small, large = P.DbShape(6, 4), P.DbShape(7, 5)
    cl = C.Client(p, seed=85)
    with SpiralGPU(p, max_batch=1) as gpu:
        gpu.set_client_keys(1, cl.public_keys(7, 5))
        rs = C.random_records(small, p, seed=86)
        rl = C.random_records(large, p, seed=87)
        gpu.load_db(1, rs, small.nu1, small.nu2)
        for i in (1, 2, 3):                   # plain, captured, replayed
            assert np.array_equal(cl.decode(gpu.answer(1, 1, cl.query(small, i))), rs[i])
        gpu.load_db(2, rl, large.nu1, large.nu2)
        assert np.array_equal(cl.decode(gpu.answer(1, 2, cl.query(large, 9))), rl[9])   # slots grow
        for i in (4, 5, 6):
            assert np.array_equal(cl.decode(gpu.answer(1, 1, cl.query(small, i))), rs[i])


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


@pytest.mark.parametrize("variant", [1, 2, 3])
def test_batch_many_columns(variant):
    """nu2 = 10 (1024 columns, 32 blocks of 128 combos): batched multiply grids
    and 10 fold levels; each result decodes and equals the query answered
    alone."""
    p = P.PARAMS
    sh = P.DbShape(7, 10)
    recs = C.random_records(sh, p, seed=91)
    cl = C.Client(p, seed=92)
    with SpiralGPU(p, max_batch=6) as gpu:
        gpu.set_client_keys(1, cl.public_keys(7, 10))
        gpu.load_db(1, recs, sh.nu1, sh.nu2)
        idx = [0, 77, 5000, sh.num_records - 1, 123456, 9]
        qs = [cl.query(sh, i) for i in idx]
        alone = [gpu.answer(1, 1, q) for q in qs]
        for i, r in zip(idx, alone):
            assert np.array_equal(cl.decode(r), recs[i])
        gpu.set_db_mul_variant(variant)
        gpu.stats_reset()
        batch = gpu.answer_batch([(1, 1, q) for q in qs])
        assert gpu.stats()["db_mul_by_variant"][variant - 1] == 1
        for x, y in zip(batch, alone):
            assert np.array_equal(x, y)


def test_serving_mixed_shapes_two_lanes():
    p = P.PARAMS
    shapes = [P.DbShape(7, 10), P.SHAPE_8MIB, P.DbShape(6, 4)]
    recs = [C.random_records(s, p, seed=93 + k) for k, s in enumerate(shapes)]
    cl = C.Client(p, seed=96)
    with SpiralGPU(p, max_batch=8) as gpu:
        gpu.set_client_keys(1, cl.public_keys(7, 10))
        for k, (s, r) in enumerate(zip(shapes, recs)):
            gpu.load_db(k, r, s.nu1, s.nu2)
        rng = np.random.default_rng(97)
        reqs, checks = [], []
        for _ in range(48):
            k = int(rng.integers(0, 3))
            i = int(rng.integers(0, shapes[k].num_records))
            reqs.append((1, k, cl.query(shapes[k], i)))
            checks.append((k, i))
        with Server(gpu, lanes=2) as srv:
            res = poisson_load(srv, reqs, rate_qps=20000.0, seed=4)
        bad = [n for n, (r, (k, i)) in enumerate(zip(res["responses"], checks))
               if not np.array_equal(cl.decode(r), recs[k][i])]
        assert not bad, f"{len(bad)} of {len(reqs)} responses wrong: {[(n, checks[n]) for n in bad[:10]]}"


def test_invalid_shape_rejected():
    """2^nu1 < t_gsw*nu2: the GSW-bit encodings would not fit the odd
    expansion outputs; the library refuses the database."""
    with SpiralGPU(P.PARAMS) as gpu:
        with pytest.raises(SpiralError) as e:
            gpu.load_db(1, np.zeros((1 << 14, 4, 2048), np.uint8), 3, 11)
        assert e.value.code == 6


def test_production_parameter_set():
    """The larger parameter set of gpu-pir/params.cuh:57-62 (t_exp_left = 16,
    t_exp_right = 56, t_gsw = 7, t_conv = 4, nu1 = 10, nu2 = 4: 1024 rows,
    11 expansion rounds, 1-bit right-branch digits): answers alone and in a
    batch are identical and decode to the records."""
    p = P.SpiralParams(n=2, pt_bits=8, t_exp_left=16, t_exp_right=56, t_gsw=7, t_conv=4, q2_bits=22)
    sh = P.DbShape(10, 4)
    recs = C.random_records(sh, p, seed=111)
    cl = C.Client(p, seed=112)
    with SpiralGPU(p, max_batch=4) as gpu:
        gpu.set_client_keys(1, cl.public_keys(sh.nu1, sh.nu2))
        gpu.load_db(1, recs, sh.nu1, sh.nu2)
        idx = [0, 12345, sh.num_records - 1, 777]
        qs = [cl.query(sh, i) for i in idx]
        alone = [gpu.answer(1, 1, q) for q in qs]
        for i, r in zip(idx, alone):
            assert np.array_equal(cl.decode(r), recs[i])
        for x, y in zip(gpu.answer_batch([(1, 1, q) for q in qs]), alone):
            assert np.array_equal(x, y)
