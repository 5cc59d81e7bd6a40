"""sp_fold_noalloc: the fold for callers that cannot allocate device memory
(inside a stream capture, under another allocator, or after a start-up-only
allocation phase).  It must give exactly sp_fold's result, call after call,
from its fixed library-owned device array, and refuse inputs larger than that
array.  Collected last so that a stop-at-first-failure run has run every other
test before it."""
import numpy as np
import pytest

from golden import cases, seeded
from spiralpir import params as P
from spiralpir.lib import SpiralError, SpiralGPU

pytestmark = pytest.mark.gpu


def test_fold_noalloc_matches_fold_twice():
    with SpiralGPU(P.PARAMS) as gpu:
        x = cases.inputs("fold")
        want = gpu.fold(x["cts"], x["V"], x["nu2"])
        for _ in range(2):      # the array keeps the previous call's contents
            got = gpu.fold_noalloc(x["cts"], x["V"], x["nu2"])
            assert np.array_equal(got, want)
        other = seeded.raw(777, (4, 8, 2))
        assert np.array_equal(gpu.fold_noalloc(other, x["V"], x["nu2"]), gpu.fold(other, x["V"], x["nu2"]))


def test_fold_noalloc_rejects_inputs_beyond_its_scratch():
    with SpiralGPU(P.PARAMS) as gpu:
        nu2 = 6     # 4 * 64 * 32 KiB = 8 MiB of ciphertexts alone
        cts = np.zeros((4, 1 << nu2, 2, 2048), dtype=np.uint64)
        gsw = np.zeros((nu2, 2, 14, 2, 2048), dtype=np.uint64)
        with pytest.raises(SpiralError) as e:
            gpu.fold_noalloc(cts, gsw, nu2)
        assert e.value.code == 1 and "scratch" in str(e.value)
