"""The answer path across parameter sets at the edges of the supported
range (gadget lengths 3 and 56, 1- and 4-bit plaintexts, n = 1, 2 and 4,
q2_bits from pt_bits + 2 to 32), on small shapes: the GPU response equals
the oracle's bit for bit.  Whether a record decodes depends on the noise
budget of the set, so decoding is checked only for the sets that have one."""
import numpy as np
import pytest

import oracle as O
from spiralpir import client as C
from spiralpir import params as P
from spiralpir.lib import SpiralGPU

pytestmark = pytest.mark.gpu

SETS = [
    # (params, shape, decodes)
    (P.SpiralParams(n=1, pt_bits=4, t_exp_left=3, t_exp_right=5, t_gsw=3, t_conv=3, q2_bits=6),
     P.DbShape(5, 3), False),
    (P.SpiralParams(n=2, pt_bits=1, t_exp_left=56, t_exp_right=56, t_gsw=28, t_conv=56, q2_bits=22),
     P.DbShape(6, 2), True),
    (P.SpiralParams(n=2, pt_bits=8, t_exp_left=16, t_exp_right=8, t_gsw=8, t_conv=8, q2_bits=32),
     P.DbShape(5, 3), True),
    (P.SpiralParams(n=1, pt_bits=4, t_exp_left=8, t_exp_right=8, t_gsw=4, t_conv=4, q2_bits=28),
     P.DbShape(5, 3), True),
    # n = 4: 16 plaintext polynomials per record, a 5 x 4 packed response;
    # 128 combos per block at nu2 = 3, the tensor-core shape
    (P.SpiralParams(n=4, pt_bits=8, t_exp_left=8, t_exp_right=8, t_gsw=7, t_conv=4, q2_bits=22),
     P.DbShape(7, 3), True),
]


@pytest.mark.parametrize("k", range(len(SETS)))
def test_param_set_matches_oracle(k):
    p, sh, decodes = SETS[k]
    recs = C.random_records(sh, p, seed=500 + k)
    cl = C.Client(p, seed=510 + k)
    keys = cl.public_keys(sh.nu1, sh.nu2)
    db = O.db_encode(recs, p.n, sh.nu1, sh.nu2, p.pt_bits)
    with SpiralGPU(p, max_batch=2) as gpu:
        gpu.set_client_keys(1, keys)
        gpu.load_db(1, recs, sh.nu1, sh.nu2)
        idx = [0, sh.num_records - 1]
        qs = [cl.query(sh, i) for i in idx]
        alone = [gpu.answer(1, 1, q) for q in qs]
        batch = gpu.answer_batch([(1, 1, q) for q in qs])
    for i, q, r, b in zip(idx, qs, alone, batch):
        ref = O.answer(db, q, keys.exp_left, keys.exp_right, keys.conv, keys.pack, n=p.n, nu1=sh.nu1,
                       nu2=sh.nu2, pt_bits=p.pt_bits, q2_bits=p.q2_bits, t_left=p.t_exp_left,
                       t_right=p.t_exp_right, t_gsw=p.t_gsw, t_conv=p.t_conv)
        assert np.array_equal(r, ref), f"set {k}: response differs from the oracle"
        assert np.array_equal(b, r), f"set {k}: batched response differs"
        if decodes:
            assert np.array_equal(cl.decode(r), recs[i]), f"set {k}: record {i} does not decode"


def test_unsupported_n_rejected():
    """n*n must be a power of two (the combo blocks of the image): n = 3 and
    n = 5 are refused when the context is created."""
    from spiralpir.lib import SpiralError
    for n in (3, 5):
        with pytest.raises(SpiralError) as e:
            SpiralGPU(P.SpiralParams(n=n))
        assert e.value.code == 6
