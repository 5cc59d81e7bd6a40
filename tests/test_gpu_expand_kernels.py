"""The three expansion kernels on the same queries: the split kernel of
narrow rounds (digit transforms spread over 2 groups per prime and several
CTAs), the one-CTA-per-output kernel and the one-CTA-per-parent kernel
(both children from one inverse transform: the upper child's raw row 0 is
the lower child's rotated by 2^r with a sign change).  The library picks
one per round by size; SPIRALPIR_EXPAND_KERNEL forces one for every round,
so each process below runs every round, round 0 and the stop round
included, through one kernel.  Every response equals the oracle's bit for
bit, single queries and a mixed batch of two clients."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import sys
import numpy as np
sys.path[:0] = [ROOT, ROOT + "/gpu-pir_gb300"]
import oracle as O
from spiralpir import client as C
from spiralpir import params as P
from spiralpir.lib import SpiralGPU

p = P.PARAMS
for (nu1, nu2) in ((5, 3), (6, 4)):
    sh = P.DbShape(nu1, nu2)
    recs = C.random_records(sh, p, seed=700 + nu1)
    clients = [C.Client(p, seed=710 + nu1), C.Client(p, seed=720 + nu1)]
    keys = [cl.public_keys(sh.nu1, sh.nu2) for cl in clients]
    db = O.db_encode(recs, p.n, sh.nu1, sh.nu2, p.pt_bits)

    def ref(q, k):
        return O.answer(db, q, k.exp_left, k.exp_right, k.conv, k.pack, n=p.n, nu1=sh.nu1, nu2=sh.nu2,
                        pt_bits=p.pt_bits, q2_bits=p.q2_bits, t_left=p.t_exp_left, t_right=p.t_exp_right,
                        t_gsw=p.t_gsw, t_conv=p.t_conv)

    with SpiralGPU(p, max_batch=4) as gpu:
        for k, ks in enumerate(keys):
            gpu.set_client_keys(1 + k, ks)
        gpu.load_db(1, recs, sh.nu1, sh.nu2)
        idx = [1, sh.num_records - 1, 7, 11]
        reqs = [(1 + s % 2, 1, clients[s % 2].query(sh, i)) for s, i in enumerate(idx)]
        want = [ref(q, keys[c - 1]) for c, _, q in reqs]
        for (c, d, q), w in zip(reqs, want):
            assert np.array_equal(gpu.answer(c, d, q), w), (nu1, nu2)
        for got, w in zip(gpu.answer_batch(reqs), want):
            assert np.array_equal(got, w), (nu1, nu2, "batch")
print("ok")
"""


@pytest.mark.parametrize("kernel", ["split", "single", "pair"])
def test_expansion_kernel_matches_oracle(kernel):
    env = dict(os.environ, SPIRALPIR_EXPAND_KERNEL=kernel)
    r = subprocess.run([sys.executable, "-c", SCRIPT.replace("ROOT", repr(ROOT))], env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout[-2000:] + r.stderr[-4000:]
