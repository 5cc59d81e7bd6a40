"""Checked mode on the GPU (SPIRALPIR_CHECKED=1): every device allocation and
every buffer carved out of a query slot is followed by a guard region that
is verified after each synchronous call (context creation first verifies
that the check catches a flipped guard byte).  The same workload -- single
answers on two shapes, batches with each multiply variant (the tensor-core
one included), staged runs, stage entry points and the serving loop --
runs in a checked and an unchecked context: no guard may be overwritten
and every result must be identical."""
import numpy as np
import pytest

from spiralpir import client as C
from spiralpir import params as P
from spiralpir.lib import SpiralGPU
from spiralpir.serving import Server, poisson_load

pytestmark = pytest.mark.gpu

SHAPES = {1: P.SHAPE_8MIB, 2: P.DbShape(7, 5)}   # (7, 5): 128 combos, tensor-core shape


def _workload():
    p = P.PARAMS
    recs = {d: C.random_records(s, p, seed=300 + d) for d, s in SHAPES.items()}
    cl = C.Client(p, seed=310)
    keys = cl.public_keys(7, 5)   # once: key generation draws fresh errors
    rng = np.random.default_rng(311)
    reqs = []
    for k in range(8):
        d = 1 + k % 2
        i = int(rng.integers(0, SHAPES[d].num_records))
        reqs.append((d, i, cl.query(SHAPES[d], i)))
    raw = rng.integers(0, P.Q1 * P.Q2, size=(3, P.D), dtype=np.uint64)
    sh = SHAPES[2]
    sel = np.empty((sh.rows, 2, 2, P.D), dtype=np.uint64)
    sel[:, :, 0] = rng.integers(0, P.Q1, size=(sh.rows, 2, P.D))
    sel[:, :, 1] = rng.integers(0, P.Q2, size=(sh.rows, 2, P.D))
    return p, recs, cl, keys, reqs, raw, sel


def _run(checked, monkeypatch, work):
    p, recs, cl, keys, reqs, raw, sel = work
    if checked:
        monkeypatch.setenv("SPIRALPIR_CHECKED", "1")
    else:
        monkeypatch.delenv("SPIRALPIR_CHECKED", raising=False)
    out = {}
    with SpiralGPU(p, max_batch=8) as gpu:
        assert gpu.check_guards() == checked
        for d, s in SHAPES.items():
            gpu.load_db(d, recs[d], s.nu1, s.nu2)
        gpu.set_client_keys(1, keys)
        out["single"] = [gpu.answer(1, d, q) for d, _, q in reqs]
        for v in (1, 2, 3):
            gpu.set_db_mul_variant(v)
            out[f"batch{v}"] = gpu.answer_batch([(1, d, q) for d, _, q in reqs])
        gpu.set_db_mul_variant(0)
        staged = [r for r in reqs if r[0] == 2]
        for slot, (d, _, q) in enumerate(staged):
            gpu.stage_query(slot, 1, d, q)
        gpu.run_staged(len(staged))
        out["staged"] = [gpu.fetch_response(s) for s in range(len(staged))]
        out["ntt"] = gpu.ntt_fwd(raw)
        out["intt"] = gpu.ntt_inv(out["ntt"])
        out["db_mul"] = gpu.db_mul(2, sel, p.T, SHAPES[2].nu2)
        with Server(gpu, lanes=2) as srv:
            res = poisson_load(srv, [(1, d, q) for d, _, q in reqs], rate_qps=5000.0, seed=3)
        out["served"] = res["responses"]
        assert gpu.check_guards() == checked
    return out


def test_checked_mode_matches_unchecked(monkeypatch):
    work = _workload()
    plain = _run(False, monkeypatch, work)
    checked = _run(True, monkeypatch, work)
    _, recs, cl, _, reqs, raw, _ = work
    for out in (plain, checked):
        for (d, i, _), r in zip(reqs, out["single"]):
            assert np.array_equal(cl.decode(r), recs[d][i])
    assert np.array_equal(plain["intt"], raw)
    for key, a in plain.items():
        b = checked[key]
        if isinstance(a, list):
            assert len(a) == len(b) and all(np.array_equal(x, y) for x, y in zip(a, b)), key
        else:
            assert np.array_equal(a, b), key
    for key in ("batch1", "batch2", "batch3", "served"):
        for x, y in zip(plain[key], plain["single"]):
            assert np.array_equal(x, y), key
