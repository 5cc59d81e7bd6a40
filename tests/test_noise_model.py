"""The expansion noise model of spiralpir.noise against the CPU oracle's
expansion at a small shape: decrypted selector and GSW-bit noise match the
model (variance doubling per round plus the key switch's share) to within
half a bit of standard deviation, which also checks the expected messages
(a wrong message would show as noise near 2^48)."""
import math

import numpy as np

import oracle as O
from spiralpir import client as C
from spiralpir import noise as N
from spiralpir import params as P


def test_expansion_noise_matches_model_on_the_oracle():
    p, sh = P.PARAMS, P.DbShape(7, 3)
    cl = C.Client(p, seed=5)
    k = cl.public_keys(7, 3)

    class OracleExpand:
        def expand(self, cid, q, nu1, nu2):
            return O.expand(q, k.exp_left, p.t_exp_left, k.exp_right, p.t_exp_right, nu1, nu2,
                            p.t_gsw).astype(np.uint64)

    r = N.expansion_noise(OracleExpand(), cl, 0, sh, 517)
    assert abs(math.log2(r["gsw_std"]) - math.log2(r["model_gsw_std"])) < 0.5
    assert abs(math.log2(r["sel_std"]) - math.log2(r["model_sel_std"])) < 0.5
    assert r["gsw_max"] < 2 ** 30
