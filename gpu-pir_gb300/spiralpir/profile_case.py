"""Small, bounded GPU cases for profiling one kernel under ncu.

    python -m spiralpir.profile_case db_mul --nu1 9 --nu2 4 --iters 3
    python -m spiralpir.profile_case db_mul_batch --nu1 9 --nu2 5 --nq 32 --variant 3
    python -m spiralpir.profile_case answer --nu1 9 --nu2 8 --iters 2
    python -m spiralpir.profile_case batch --nu1 9 --nu2 8 --nq 32 --iters 2

db_mul: one database of the given shape (random records) and random
selectors; runs the first-dimension multiply `iters` times through
sp_db_mul.  db_mul_batch: the same for `nq` selector sets in one launch
with multiply variant `variant` (1 per-query, 2 batched integer, 3 tensor
core) through sp_db_mul_batch.  answer: a real client's queries answered `iters` times at the
given shape (expansion, conversion, multiply, fold, pack kernels).  batch:
`nq` such queries staged and answered together `iters` times (the batched
pipeline: one launch per stage for all queries).
Prints the device bytes held so that a capture stays small.
"""
from __future__ import annotations

import argparse

import numpy as np

from . import client as C
from . import params as P
from .lib import SpiralGPU


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["db_mul", "db_mul_batch", "answer", "batch"])
    ap.add_argument("--nu1", type=int, default=9)
    ap.add_argument("--nu2", type=int, default=4)
    ap.add_argument("--iters", type=int, default=3)
    ap.add_argument("--nq", type=int, default=32)
    ap.add_argument("--variant", type=int, default=3)
    a = ap.parse_args()
    p = P.PARAMS
    sh = P.DbShape(a.nu1, a.nu2)
    recs = C.random_records(sh, p, seed=1)
    with SpiralGPU(p, max_batch=max(1, a.nq if a.case == "batch" else 1)) as gpu:
        gpu.load_db(1, recs, sh.nu1, sh.nu2)
        if a.case in ("db_mul", "db_mul_batch"):
            rng = np.random.default_rng(2)
            sel = np.empty((sh.rows, 2, 2, P.D), dtype=np.uint64)
            sel[:, :, 0] = rng.integers(0, P.Q1, size=(sh.rows, 2, P.D))
            sel[:, :, 1] = rng.integers(0, P.Q2, size=(sh.rows, 2, P.D))
            if a.case == "db_mul":
                for _ in range(a.iters):
                    gpu.db_mul(1, sel, p.T, sh.nu2)
            else:
                sels = np.ascontiguousarray(np.broadcast_to(sel, (a.nq,) + sel.shape))
                gpu.set_db_mul_variant(a.variant)
                for _ in range(a.iters):
                    gpu.db_mul_batch(1, sels, p.T, sh.nu2)
        elif a.case == "answer":
            cl = C.Client(p, seed=3)
            gpu.set_client_keys(1, cl.public_keys(sh.nu1, sh.nu2))
            q = cl.query(sh, 5)
            for _ in range(a.iters):
                r = gpu.answer(1, 1, q)
            assert np.array_equal(cl.decode(r), recs[5])
        else:
            cl = C.Client(p, seed=3)
            gpu.set_client_keys(1, cl.public_keys(sh.nu1, sh.nu2))
            q = cl.query(sh, 5)
            for s in range(a.nq):
                gpu.stage_query(s, 1, 1, q)
            for _ in range(a.iters):
                gpu.run_staged(a.nq)
            assert np.array_equal(cl.decode(gpu.fetch_response(a.nq - 1)), recs[5])
        print(f"case {a.case} nu1={sh.nu1} nu2={sh.nu2}: device bytes held {gpu.hbm_used() / 2**20:.0f} MiB")


if __name__ == "__main__":
    main()
