"""Failure detection on the GPU without a fault: a device barrier wait that
nothing completes gives up after its limit, the kernel returns with the
error flag set, the call reports SP_ERR_DEVICE, and the context keeps
answering correctly afterwards."""
import time

import numpy as np
import pytest

from spiralpir import client as C
from spiralpir import params as P
from spiralpir.lib import SpiralError, SpiralGPU

pytestmark = pytest.mark.gpu


def test_bounded_wait_runs_out_and_context_survives():
    p, sh = P.PARAMS, P.SHAPE_8MIB
    recs = C.random_records(sh, p, seed=401)
    cl = C.Client(p, seed=402)
    with SpiralGPU(p) as gpu:
        gpu.set_client_keys(1, cl.public_keys(sh.nu1, sh.nu2))
        gpu.load_db(1, recs, sh.nu1, sh.nu2)
        assert np.array_equal(cl.decode(gpu.answer(1, 1, cl.query(sh, 5))), recs[5])
        for limit_ms in (20, 100):
            t0 = time.perf_counter()
            with pytest.raises(SpiralError) as e:
                gpu.wait_probe(limit_ms)
            dt = time.perf_counter() - t0
            assert e.value.code == 5 and "bounded wait" in str(e.value)
            assert limit_ms / 1e3 <= dt < 5.0
            # the flag was taken: the context answers again, bit-exact
            for i in (0, 777, sh.num_records - 1):
                assert np.array_equal(cl.decode(gpu.answer(1, 1, cl.query(sh, i))), recs[i])
        with pytest.raises(SpiralError) as e:
            gpu.wait_probe(0)
        assert e.value.code == 1
