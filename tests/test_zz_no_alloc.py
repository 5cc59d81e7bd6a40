"""sp_fold_noalloc: the fold for callers that cannot allocate device memory
(a process whose GPU memory another allocator already holds, or a service
that allocates only at start-up).  It must give exactly sp_fold's result,
call after call, from its fixed library-owned device array, leave the
device's free memory unchanged, and refuse inputs larger than that array.
Collected last so that a stop-at-first-failure run has run every other test
before it."""
import ctypes

import numpy as np
import pytest

from golden import cases, seeded
from spiralpir import params as P
from spiralpir.lib import SpiralError, SpiralGPU

pytestmark = pytest.mark.gpu


def _free_device_bytes() -> int:
    """cudaMemGetInfo's free bytes of the current context (driver API)."""
    cuda = ctypes.CDLL("libcuda.so.1")
    free, total = ctypes.c_size_t(), ctypes.c_size_t()
    rc = cuda.cuMemGetInfo_v2(ctypes.byref(free), ctypes.byref(total))
    assert rc == 0, f"cuMemGetInfo failed ({rc})"
    return free.value


def test_fold_noalloc_matches_fold_twice():
    with SpiralGPU(P.PARAMS) as gpu:
        x = cases.inputs("fold")
        want = gpu.fold(x["cts"], x["V"], x["nu2"])
        for _ in range(2):      # the array keeps the previous call's contents
            got = gpu.fold_noalloc(x["cts"], x["V"], x["nu2"])
            assert np.array_equal(got, want)
        other = seeded.raw(777, (4, 8, 2))
        assert np.array_equal(gpu.fold_noalloc(other, x["V"], x["nu2"]), gpu.fold(other, x["V"], x["nu2"]))


def test_fold_noalloc_allocates_nothing():
    """After a first call (which resolves the array's address), further
    calls leave the device's free memory exactly as it was."""
    with SpiralGPU(P.PARAMS) as gpu:
        x = cases.inputs("fold")
        want = gpu.fold(x["cts"], x["V"], x["nu2"])
        gpu.fold_noalloc(x["cts"], x["V"], x["nu2"])
        before = _free_device_bytes()
        for _ in range(3):
            assert np.array_equal(gpu.fold_noalloc(x["cts"], x["V"], x["nu2"]), want)
        assert _free_device_bytes() == before


def test_fold_noalloc_size_limit_boundary():
    """T = 4: nu2 = 4 needs 2 MiB of ciphertexts + 4 * 7 * 192 KiB of GSW
    ciphertexts (7.25 MiB) and runs; nu2 = 5 needs 10.56 MiB and is refused."""
    with SpiralGPU(P.PARAMS) as gpu:
        t = gpu.params.t_gsw
        nu2 = 4
        cts = seeded.raw(901, (4, 1 << nu2, 2))
        gsw = seeded.residues(902, (nu2, 2, 2 * t)).astype(np.uint64)
        assert np.array_equal(gpu.fold_noalloc(cts, gsw, nu2), gpu.fold(cts, gsw, nu2))
        nu2 = 5
        cts = np.zeros((4, 1 << nu2, 2, 2048), dtype=np.uint64)
        gsw = np.zeros((nu2, 2, 2 * t, 2, 2048), dtype=np.uint64)
        with pytest.raises(SpiralError) as e:
            gpu.fold_noalloc(cts, gsw, nu2)
        assert e.value.code == 1 and "scratch" in str(e.value)


def test_fold_noalloc_rejects_inputs_beyond_its_scratch():
    with SpiralGPU(P.PARAMS) as gpu:
        nu2 = 6     # 4 * 64 * 32 KiB = 8 MiB of ciphertexts alone
        cts = np.zeros((4, 1 << nu2, 2, 2048), dtype=np.uint64)
        gsw = np.zeros((nu2, 2, 14, 2, 2048), dtype=np.uint64)
        with pytest.raises(SpiralError) as e:
            gpu.fold_noalloc(cts, gsw, nu2)
        assert e.value.code == 1 and "scratch" in str(e.value)


def test_fold_noalloc_checked_mode(monkeypatch):
    """In checked mode the guard after the call's data in the array is
    verified; a correct fold leaves it intact and gives sp_fold's result."""
    monkeypatch.setenv("SPIRALPIR_CHECKED", "1")
    with SpiralGPU(P.PARAMS) as gpu:
        x = cases.inputs("fold")
        want = gpu.fold(x["cts"], x["V"], x["nu2"])
        for _ in range(2):
            assert np.array_equal(gpu.fold_noalloc(x["cts"], x["V"], x["nu2"]), want)
