"""Autotuning of the narrow launches' split schedule: every schedule (forced
or tuned) answers with identical bytes, the tuner records the batch classes
it tuned with each candidate's time and its choice, and forcing rejects bad
values."""
import numpy as np
import pytest

from spiralpir import client as C
from spiralpir import params as P
from spiralpir.lib import SPLIT_AUTO, SPLIT_NONE, SpiralError, SpiralGPU

pytestmark = pytest.mark.gpu


def test_split_schedules_give_identical_answers():
    p, sh = P.PARAMS, P.SHAPE_8MIB
    cl = C.Client(p, seed=81)
    keys = cl.public_keys(sh.nu1, sh.nu2)
    recs = C.random_records(sh, p, seed=82)
    qs = [cl.query(sh, i) for i in (3, 500, 1023)]
    with SpiralGPU(p, max_batch=4) as gpu:
        gpu.set_client_keys(1, keys)
        gpu.load_db(1, recs, sh.nu1, sh.nu2)
        ref = [gpu.answer(1, 1, q) for q in qs]                 # autotuned (default)
        ref_batch = gpu.answer_batch([(1, 1, q) for q in qs])
        report = gpu.tuning_report()
        assert "plan class nq<=1 " in report and "plan class nq<=4 " in report and "chosen" in report
        for shift in (SPLIT_NONE, -1, 0, 1, 2):
            gpu.set_split_schedule(shift)
            for q, r in zip(qs, ref):
                assert np.array_equal(gpu.answer(1, 1, q), r), shift
            for x, y in zip(gpu.answer_batch([(1, 1, q) for q in qs]), ref_batch):
                assert np.array_equal(x, y), shift
        gpu.set_split_schedule(SPLIT_AUTO)
        assert np.array_equal(cl.decode(gpu.answer(1, 1, qs[0])), recs[3])
        with pytest.raises(SpiralError):
            gpu.set_split_schedule(9)
