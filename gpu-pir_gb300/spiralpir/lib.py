"""ctypes binding of libspiralpir.so (include/spiralpir.h).

`SpiralGPU` owns one context.  Every call goes to the CUDA library; there is
no CPU fallback: constructing a context without the built library or
without a GPU raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .client import PublicKeys, as_u64
from .params import D, SpiralParams

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libspiralpir.so")
HEADER = os.path.join(os.path.dirname(os.path.dirname(_HERE)), "include", "spiralpir.h")

SP_OK = 0
SPLIT_AUTO = 127     # sp_set_split_schedule: autotune per batch class
SPLIT_NONE = -16     # one CTA per item in every narrow launch
ERRORS = {1: "INVALID", 2: "CUDA", 3: "NOMEM", 4: "NOT_FOUND", 5: "DEVICE", 6: "UNSUPPORTED", 7: "IO"}


class SpiralError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class SpParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int32) for n in
                ("n", "pt_bits", "t_exp_left", "t_exp_right", "t_gsw", "t_conv", "q2_bits", "max_batch")]


class SpStats(ctypes.Structure):
    _fields_ = [("answers", ctypes.c_uint64), ("launches", ctypes.c_uint64),
                ("ms_expand", ctypes.c_double), ("ms_convert", ctypes.c_double),
                ("ms_db_mul", ctypes.c_double), ("ms_fold", ctypes.c_double),
                ("ms_pack", ctypes.c_double), ("ms_total", ctypes.c_double),
                ("db_mul_calls", ctypes.c_uint64), ("db_mul_bytes", ctypes.c_uint64),
                ("db_mul_by_variant", ctypes.c_uint64 * 3)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["db_mul_by_variant"] = list(self.db_mul_by_variant)
        return d


class SpRequest(ctypes.Structure):
    _fields_ = [("client_id", ctypes.c_int32), ("db_id", ctypes.c_int32),
                ("query", ctypes.c_void_p), ("response", ctypes.c_void_p),
                ("response_len", ctypes.c_uint64), ("status", ctypes.c_int32)]


_lib = None

_P = ctypes.c_void_p
_I = ctypes.c_int32
_U32 = ctypes.c_uint32
_U64 = ctypes.c_uint64
_SIGS = {
    "sp_ctx_create": [ctypes.POINTER(SpParams), _U64, ctypes.POINTER(_P)],
    "sp_ctx_destroy": [_P],
    "sp_last_error": [ctypes.c_char_p, ctypes.c_size_t],
    "sp_response_bytes": [_P, ctypes.POINTER(_U64)],
    "sp_hbm_used": [_P, ctypes.POINTER(_U64)],
    "sp_db_load_plain": [_P, _I, _P, _U64, _I, _I],
    "sp_db_load_ntt": [_P, _I, _P, _I, _I],
    "sp_db_unload": [_P, _I],
    "sp_client_set_keys": [_P, _I, _P, _I, _P, _I, _P, _P],
    "sp_client_set_keys_seeded": [_P, _I, _P, _P, _I, _P, _I, _P, _P],
    "sp_set_split_schedule": [_P, _I],
    "sp_tuning_report": [_P, _P, _U64],
    "sp_client_evict": [_P, _I],
    "sp_answer": [_P, _I, _I, _P, _P, _U64],
    "sp_answer_batch": [_P, _I, ctypes.POINTER(SpRequest)],
    "sp_stage_query": [_P, _I, _I, _I, _P],
    "sp_run_staged": [_P, _I],
    "sp_fetch_response": [_P, _I, _P, _U64],
    "sp_time_staged": [_P, _I, _I, ctypes.POINTER(ctypes.c_double)],
    "sp_set_db_mul_variant": [_P, _I],
    "sp_serve_start": [_P, _I],
    "sp_serve_stop": [_P],
    "sp_submit": [_P, ctypes.POINTER(SpRequest), ctypes.POINTER(_U64)],
    "sp_poll": [_P, _U64, ctypes.POINTER(_I), ctypes.POINTER(_I)],
    "sp_wait": [_P, _U64, ctypes.POINTER(_I)],
    "sp_wait_timed": [_P, _U64, ctypes.POINTER(_I), ctypes.POINTER(ctypes.c_double)],
    "sp_serve_stats": [_P, ctypes.POINTER(_U64), ctypes.POINTER(_U64), ctypes.POINTER(_U64)],
    "sp_stats": [_P, ctypes.POINTER(SpStats)],
    "sp_stats_reset": [_P],
    "sp_time_db_mul": [_P, _I, _I, _I, ctypes.POINTER(ctypes.c_double)],
    "sp_ntt_fwd": [_P, _P, _P, _U64],
    "sp_ntt_inv": [_P, _P, _P, _U64],
    "sp_automorph": [_P, _P, _P, _U64, _U32],
    "sp_expand": [_P, _I, _P, _I, _I, _I, _P],
    "sp_regev_to_gsw": [_P, _I, _P, _I, _P],
    "sp_gsw_neg": [_P, _P, _I, _P],
    "sp_db_mul": [_P, _I, _P, _P],
    "sp_db_mul_batch": [_P, _I, _I, _P, _P],
    "sp_set_graphs": [_P, _I],
    "sp_set_stage_timing": [_P, _I],
    "sp_db_save": [_P, _I, ctypes.c_char_p],
    "sp_db_restore": [_P, _I, ctypes.c_char_p],
    "sp_fold": [_P, _P, _P, _I, _I, _P],
    "sp_fold_noalloc": [_P, _P, _P, _I, _I, _P],
    "sp_pack": [_P, _I, _P, _P, _U64],
    "sp_check_guards": [_P, _P],
    "sp_wait_probe": [_P, _I],
}


def exported_symbols() -> list[str]:
    return list(_SIGS)


def load(path: str = LIB_PATH):
    """Load the CUDA library, building it first when the shared object is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        from . import build
        build.build()
    lib = ctypes.CDLL(path)
    for name, args in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    _lib = lib
    return lib


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def _check(rc: int) -> None:
    if rc != SP_OK:
        buf = ctypes.create_string_buffer(512)
        _lib.sp_last_error(buf, 512)
        raise SpiralError(rc, buf.value.decode(errors="replace"))


def _u64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint64)


class SpiralGPU:
    """One answer-path context on the current CUDA device."""

    def __init__(self, params: SpiralParams, hbm_budget_bytes: int = 0, max_batch: int = 1):
        self.lib = load()
        self.params = params
        p = SpParams(params.n, params.pt_bits, params.t_exp_left, params.t_exp_right, params.t_gsw,
                     params.t_conv, params.q2_bits, max_batch)
        h = _P()
        _check(self.lib.sp_ctx_create(ctypes.byref(p), hbm_budget_bytes, ctypes.byref(h)))
        self.h = h
        rb = _U64()
        _check(self.lib.sp_response_bytes(self.h, ctypes.byref(rb)))
        self.response_bytes = rb.value
        self.max_batch = max_batch

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.sp_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- resources ---------------------------------------------------------
    def check_guards(self) -> bool:
        """Verify the guard regions now; True when the context runs in
        checked mode (SPIRALPIR_CHECKED=1 at creation).  Raises SpiralError
        when a guard was overwritten."""
        on = _I()
        _check(self.lib.sp_check_guards(self.h, ctypes.byref(on)))
        return bool(on.value)

    def wait_probe(self, limit_ms: int) -> None:
        """Run the bounded-wait failure path once: raises SpiralError
        (SP_ERR_DEVICE) after about limit_ms; the context stays usable."""
        _check(self.lib.sp_wait_probe(self.h, limit_ms))

    def hbm_used(self) -> int:
        v = _U64()
        _check(self.lib.sp_hbm_used(self.h, ctypes.byref(v)))
        return v.value

    def load_db(self, db_id: int, records: np.ndarray, nu1: int, nu2: int) -> None:
        rec = np.ascontiguousarray(records, dtype=np.uint8)
        _check(self.lib.sp_db_load_plain(self.h, db_id, _ptr(rec), rec.shape[0], nu1, nu2))

    def load_db_ntt(self, db_id: int, planes: np.ndarray, nu1: int, nu2: int) -> None:
        pl = np.ascontiguousarray(planes, dtype=np.uint32)
        _check(self.lib.sp_db_load_ntt(self.h, db_id, _ptr(pl), nu1, nu2))

    def save_db(self, db_id: int, path: str) -> None:
        """Write database `db_id`'s encoded device image to `path`."""
        _check(self.lib.sp_db_save(self.h, db_id, os.fsencode(path)))

    def restore_db(self, db_id: int, path: str) -> None:
        """Load an image written by save_db as database `db_id` (no encode)."""
        _check(self.lib.sp_db_restore(self.h, db_id, os.fsencode(path)))

    def unload_db(self, db_id: int) -> None:
        _check(self.lib.sp_db_unload(self.h, db_id))

    def set_client_keys(self, client_id: int, keys: PublicKeys) -> None:
        left, right = as_u64(keys.exp_left), as_u64(keys.exp_right)
        conv, pack = as_u64(keys.conv), as_u64(keys.pack)
        _check(self.lib.sp_client_set_keys(self.h, client_id, _ptr(left), left.shape[0], _ptr(right),
                                           right.shape[0], _ptr(conv), _ptr(pack)))

    def set_client_keys_seeded(self, client_id: int, seed: bytes, keys: PublicKeys) -> None:
        """Register keys whose row 0 (every key matrix) the library expands
        from `seed` on the device; only the other rows of `keys` are sent."""
        if len(seed) != 32:
            raise ValueError("the seed is 32 bytes")
        sd = np.frombuffer(bytes(seed), dtype=np.uint8).copy()
        left = as_u64(keys.exp_left[:, 1])
        right = as_u64(keys.exp_right[:, 1])
        conv = as_u64(keys.conv[1])
        pack = as_u64(keys.pack[:, 1:])
        _check(self.lib.sp_client_set_keys_seeded(self.h, client_id, _ptr(sd), _ptr(left), left.shape[0],
                                                  _ptr(right), right.shape[0], _ptr(conv), _ptr(pack)))

    def set_split_schedule(self, shift: int) -> None:
        """Force the narrow launches' split schedule (SPLIT_NONE, or a shift
        in [-4, 4]) or autotune it per batch class (SPLIT_AUTO, the default)."""
        _check(self.lib.sp_set_split_schedule(self.h, int(shift)))

    def tuning_report(self) -> str:
        buf = ctypes.create_string_buffer(1 << 16)
        _check(self.lib.sp_tuning_report(self.h, buf, len(buf)))
        return buf.value.decode()

    def evict_client(self, client_id: int) -> None:
        _check(self.lib.sp_client_evict(self.h, client_id))

    # -- answering -----------------------------------------------------------
    def answer(self, client_id: int, db_id: int, query: np.ndarray, out: np.ndarray | None = None) -> np.ndarray:
        q = _u64(query)
        resp = out if out is not None else np.empty(self.response_bytes, dtype=np.uint8)
        _check(self.lib.sp_answer(self.h, client_id, db_id, _ptr(q), _ptr(resp), resp.nbytes))
        return resp

    def answer_batch(self, requests: list[tuple[int, int, np.ndarray]]) -> list[np.ndarray]:
        qs = [_u64(q) for _, _, q in requests]
        outs = [np.empty(self.response_bytes, dtype=np.uint8) for _ in requests]
        arr = (SpRequest * len(requests))()
        for i, ((cid, did, _), q, o) in enumerate(zip(requests, qs, outs)):
            arr[i] = SpRequest(cid, did, _ptr(q), _ptr(o), o.nbytes, 0)
        _check(self.lib.sp_answer_batch(self.h, len(requests), arr))
        return outs

    def stage_query(self, slot: int, client_id: int, db_id: int, query: np.ndarray) -> None:
        q = _u64(query)
        _check(self.lib.sp_stage_query(self.h, slot, client_id, db_id, _ptr(q)))

    def run_staged(self, count: int) -> None:
        _check(self.lib.sp_run_staged(self.h, count))

    def time_staged(self, count: int, iters: int) -> float:
        ms = ctypes.c_double()
        _check(self.lib.sp_time_staged(self.h, count, iters, ctypes.byref(ms)))
        return ms.value

    def fetch_response(self, slot: int) -> np.ndarray:
        resp = np.empty(self.response_bytes, dtype=np.uint8)
        _check(self.lib.sp_fetch_response(self.h, slot, _ptr(resp), resp.nbytes))
        return resp

    def set_db_mul_variant(self, variant: int) -> None:
        """0 = autotune, 1 = per-query streaming multiply, 2 = batched integer
        multiply, 3 = tensor-core multiply."""
        _check(self.lib.sp_set_db_mul_variant(self.h, variant))

    def set_graphs(self, on: bool) -> None:
        """Replay the answer pipeline as CUDA graphs (default) or launch its
        kernels one by one."""
        _check(self.lib.sp_set_graphs(self.h, 1 if on else 0))

    def set_stage_timing(self, on: bool) -> None:
        """Per-stage device time in stats() (ms_expand .. ms_pack): an event
        between every two stages of each answer run (off by default, when
        only ms_total is measured and the stages run as dependent launches)."""
        _check(self.lib.sp_set_stage_timing(self.h, 1 if on else 0))

    def stats(self) -> dict:
        s = SpStats()
        _check(self.lib.sp_stats(self.h, ctypes.byref(s)))
        return s.as_dict()

    def stats_reset(self) -> None:
        _check(self.lib.sp_stats_reset(self.h))

    def time_db_mul(self, db_id: int, nq: int, iters: int) -> float:
        ms = ctypes.c_double()
        _check(self.lib.sp_time_db_mul(self.h, db_id, nq, iters, ctypes.byref(ms)))
        return ms.value

    # -- stages (fixture layouts, uint64) ----------------------------------
    def ntt_fwd(self, raw: np.ndarray) -> np.ndarray:
        raw = _u64(raw)
        n = raw.size // D
        out = np.empty(raw.shape[:-1] + (2, D), dtype=np.uint64)
        _check(self.lib.sp_ntt_fwd(self.h, _ptr(raw), _ptr(out), n))
        return out

    def ntt_inv(self, crt: np.ndarray) -> np.ndarray:
        crt = _u64(crt)
        n = crt.size // (2 * D)
        out = np.empty(crt.shape[:-2] + (D,), dtype=np.uint64)
        _check(self.lib.sp_ntt_inv(self.h, _ptr(crt), _ptr(out), n))
        return out

    def automorph(self, raw: np.ndarray, t: int) -> np.ndarray:
        raw = _u64(raw)
        out = np.empty_like(raw)
        _check(self.lib.sp_automorph(self.h, _ptr(raw), _ptr(out), raw.size // D, t))
        return out

    def expand(self, client_id: int, query: np.ndarray, nu1: int, nu2: int, rounds: int = 0) -> np.ndarray:
        q = _u64(query)
        r = rounds or self.params.g(nu1, nu2)
        out = np.empty(((1 << r), 2, 2, D), dtype=np.uint64)
        _check(self.lib.sp_expand(self.h, client_id, _ptr(q), nu1, nu2, rounds, _ptr(out)))
        return out

    def regev_to_gsw(self, client_id: int, regev: np.ndarray, nu2: int) -> np.ndarray:
        r = _u64(regev)
        out = np.empty((nu2, 2, 2 * self.params.t_gsw, 2, D), dtype=np.uint64)
        _check(self.lib.sp_regev_to_gsw(self.h, client_id, _ptr(r), nu2, _ptr(out)))
        return out

    def gsw_neg(self, gsw: np.ndarray) -> np.ndarray:
        g = _u64(gsw)
        out = np.empty_like(g)
        count = g.size // (2 * 2 * self.params.t_gsw * 2 * D)
        _check(self.lib.sp_gsw_neg(self.h, _ptr(g), count, _ptr(out)))
        return out

    def db_mul(self, db_id: int, sel: np.ndarray, T: int, nu2: int) -> np.ndarray:
        s = _u64(sel)
        out = np.empty((T, 1 << nu2, 2, 2, D), dtype=np.uint64)
        _check(self.lib.sp_db_mul(self.h, db_id, _ptr(s), _ptr(out)))
        return out

    def db_mul_batch(self, db_id: int, sels: np.ndarray, T: int, nu2: int) -> np.ndarray:
        """sels [nq][2^nu1][2][2][D] -> [nq][T][2^nu2][2][2][D] with the forced
        (or autotuned) multiply variant."""
        s = _u64(sels)
        nq = s.shape[0]
        out = np.empty((nq, T, 1 << nu2, 2, 2, D), dtype=np.uint64)
        _check(self.lib.sp_db_mul_batch(self.h, db_id, nq, _ptr(s), _ptr(out)))
        return out

    def fold(self, cts: np.ndarray, gsw: np.ndarray, nu2: int) -> np.ndarray:
        c = _u64(cts)
        g = _u64(gsw)
        T = c.size // ((1 << nu2) * 2 * D)
        out = np.empty((T, 2, D), dtype=np.uint64)
        _check(self.lib.sp_fold(self.h, _ptr(c), _ptr(g), T, nu2, _ptr(out)))
        return out

    def fold_noalloc(self, cts: np.ndarray, gsw: np.ndarray, nu2: int) -> np.ndarray:
        """sp_fold without device allocation (fixed library-owned scratch)."""
        c = _u64(cts)
        g = _u64(gsw)
        T = c.size // ((1 << nu2) * 2 * D)
        out = np.empty((T, 2, D), dtype=np.uint64)
        _check(self.lib.sp_fold_noalloc(self.h, _ptr(c), _ptr(g), T, nu2, _ptr(out)))
        return out

    def pack(self, client_id: int, cts: np.ndarray) -> np.ndarray:
        c = _u64(cts)
        out = np.empty(self.response_bytes, dtype=np.uint8)
        _check(self.lib.sp_pack(self.h, client_id, _ptr(c), _ptr(out), out.nbytes))
        return out


def header_symbols(path: str = HEADER) -> list[str]:
    """Function names declared in include/spiralpir.h."""
    import re
    text = open(path).read()
    return sorted(set(re.findall(r"^int\s+(sp_\w+)\s*\(", text, flags=re.M)))
