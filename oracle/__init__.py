"""CPU oracle for the Spiral PIR answer path (test infrastructure only).

This package is the checker.  Only ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py``'s CPU-baseline leg may import it; the product library under
``gpu-pir_gb300/`` never does.  It wraps ``spiral_oracle.c`` (compiled to
``oracle/_build/liboracle.so`` by ``build()``) with numpy-facing functions.

Array layouts (numpy, C order):
  crt poly  uint32 (2, D)            residues mod q1 then q2, NTT spiral order
  raw poly  uint64 (D,)              coefficients mod q
  NTT ct    uint32 (rows, 2, D)
  raw ct    uint64 (rows, D)
  matrix    uint32 (rows, cols, 2, D)
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

D = 2048
Q1 = 268369921
Q2 = 249561089
Q = Q1 * Q2
MOD_BITS = 56

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None
_lock = threading.Lock()

_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_i = ctypes.c_int
_u32 = ctypes.c_uint32
_u64 = ctypes.c_uint64


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile; returns the library path."""
    src = os.path.join(_HERE, "spiral_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def _load():
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        build()
        lib = ctypes.CDLL(_LIB_PATH)
        sig = {
            "or_num_threads": ([], _i),
            "or_set_threads": ([_i], None),
            "or_ntt_fwd": ([_u32p, _i], None),
            "or_ntt_inv": ([_u32p, _i], None),
            "or_from_ntt": ([_u32p, _u64p], None),
            "or_to_ntt": ([_u64p, _u32p], None),
            "or_ntt_fwd_many": ([_u32p, _u64], None),
            "or_from_ntt_many": ([_u32p, _u64p, _u64], None),
            "or_to_ntt_many": ([_u64p, _u32p, _u64], None),
            "or_automorph": ([_u64p, _u64p, _u32], None),
            "or_bits_per": ([_i], _i),
            "or_expansion_g": ([_i, _i, _i], _i),
            "or_expansion_stop": ([_i, _i], _i),
            "or_neg1": ([_i, _u32p], None),
            "or_expand": ([_u32p, _u32p, _i, _u32p, _i, _i, _i, _i, _i, _u32p], None),
            "or_regev_to_gsw": ([_u32p, _u32p, _i, _i, _i, _u32p], None),
            "or_gsw_neg": ([_u32p, _i, _i, _u32p], None),
            "or_db_encode": ([_u8p, _i, _i, _i, _i, _u32p], None),
            "or_db_mul": ([_u32p, _u32p, _i, _i, _i, _u32p], None),
            "or_fold": ([_u64p, _u32p, _u32p, _i, _i], None),
            "or_fold_many": ([_u64p, _i, _u32p, _u32p, _i, _i], None),
            "or_pack": ([_u64p, _u32p, _i, _i, _u64p], None),
            "or_rescale": ([_u64, _u64, _u64], _u64),
            "or_response_bytes": ([_i, _i, _i], _u64),
            "or_encode_response": ([_u64p, _i, _i, _i, _u8p], None),
            "or_answer": ([_u32p, _i, _i, _i, _i, _i, _i, _i, _i, _i, _u32p, _u32p, _u32p,
                           _u32p, _u32p, _u8p, _u32p, _u32p, _u64p], _i),
        }
        for name, (args, res) in sig.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _lib = lib
        return lib


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def num_threads() -> int:
    return _load().or_num_threads()


def set_threads(n: int) -> None:
    _load().or_set_threads(int(n))


def bits_per(t: int) -> int:
    return _load().or_bits_per(int(t))


def expansion_g(nu1: int, nu2: int, t_gsw: int) -> int:
    return _load().or_expansion_g(nu1, nu2, t_gsw)


def expansion_stop(nu2: int, t_gsw: int) -> int:
    return _load().or_expansion_stop(nu2, t_gsw)


def ntt(raw_or_res: np.ndarray) -> np.ndarray:
    """Forward NTT of residue planes: uint32 (..., 2, D) canonical -> same shape."""
    a = _c(raw_or_res, np.uint32).copy()
    _load().or_ntt_fwd_many(a, a.size // (2 * D))
    return a


def to_ntt(raw: np.ndarray) -> np.ndarray:
    """raw uint64 (..., D) -> NTT form uint32 (..., 2, D)."""
    raw = _c(raw, np.uint64)
    out = np.empty(raw.shape[:-1] + (2, D), dtype=np.uint32)
    _load().or_to_ntt_many(raw, out, raw.size // D)
    return out


def from_ntt(a: np.ndarray) -> np.ndarray:
    """NTT form uint32 (..., 2, D) -> raw uint64 (..., D)."""
    a = _c(a, np.uint32)
    out = np.empty(a.shape[:-2] + (D,), dtype=np.uint64)
    _load().or_from_ntt_many(a, out, a.size // (2 * D))
    return out


def automorph(raw: np.ndarray, t: int) -> np.ndarray:
    raw = _c(raw, np.uint64)
    out = np.empty_like(raw)
    _load().or_automorph(raw, out, int(t))
    return out


def neg1(r: int) -> np.ndarray:
    out = np.empty((2, D), dtype=np.uint32)
    _load().or_neg1(int(r), out)
    return out


def expand(query, left, t_left, right, t_right, nu1, nu2, t_gsw, rounds=None) -> np.ndarray:
    """Coefficient expansion; returns uint32 (2^rounds, 2, 2, D)."""
    if rounds is None:
        rounds = expansion_g(nu1, nu2, t_gsw)
    out = np.empty(((1 << rounds), 2, 2, D), dtype=np.uint32)
    _load().or_expand(_c(query, np.uint32), _c(left, np.uint32), t_left, _c(right, np.uint32),
                      t_right, nu1, nu2, t_gsw, rounds, out)
    return out


def regev_to_gsw(regev, conv, nu2, t_gsw, t_conv) -> np.ndarray:
    out = np.empty((nu2, 2, 2 * t_gsw, 2, D), dtype=np.uint32)
    _load().or_regev_to_gsw(_c(regev, np.uint32), _c(conv, np.uint32), nu2, t_gsw, t_conv, out)
    return out


def gsw_neg(gsw, t) -> np.ndarray:
    gsw = _c(gsw, np.uint32)
    out = np.empty_like(gsw)
    _load().or_gsw_neg(gsw, gsw.size // (2 * 2 * t * 2 * D), t, out)
    return out


def db_encode(records: np.ndarray, n, nu1, nu2, pt_bits) -> np.ndarray:
    """uint8 records (2^(nu1+nu2), n*n, D) -> uint32 (n*n, 2^nu2, 2^nu1, 2, D)."""
    out = np.empty((n * n, 1 << nu2, 1 << nu1, 2, D), dtype=np.uint32)
    _load().or_db_encode(_c(records, np.uint8), n, nu1, nu2, pt_bits, out)
    return out


def db_mul(db, sel, T, nu1, nu2) -> np.ndarray:
    out = np.empty((T, 1 << nu2, 2, 2, D), dtype=np.uint32)
    _load().or_db_mul(_c(db, np.uint32), _c(sel, np.uint32), T, nu1, nu2, out)
    return out


def fold(cts, V, Vneg, nu2, t_gsw) -> np.ndarray:
    """cts uint64 (T, 2^nu2, 2, D) -> folded uint64 (T, 2, D)."""
    a = _c(cts, np.uint64).copy()
    T = a.size // ((1 << nu2) * 2 * D)
    _load().or_fold_many(a, T, _c(V, np.uint32), _c(Vneg, np.uint32), nu2, t_gsw)
    return a.reshape(T, 1 << nu2, 2, D)[:, 0].copy()


def pack(cts, keys, n, t_conv) -> np.ndarray:
    out = np.empty((n + 1, n, D), dtype=np.uint64)
    _load().or_pack(_c(cts, np.uint64), _c(keys, np.uint32), n, t_conv, out)
    return out


def rescale(x: int, q_in: int, q_out: int) -> int:
    return int(_load().or_rescale(int(x), int(q_in), int(q_out)))


def response_bytes(n, pt_bits, q2_bits) -> int:
    return int(_load().or_response_bytes(n, pt_bits, q2_bits))


def encode_response(packed, n, pt_bits, q2_bits) -> np.ndarray:
    out = np.zeros(response_bytes(n, pt_bits, q2_bits), dtype=np.uint8)
    _load().or_encode_response(_c(packed, np.uint64), n, pt_bits, q2_bits, out)
    return out


def answer(db, query, left, right, conv, pack_keys, *, n, nu1, nu2, pt_bits, q2_bits,
           t_left, t_right, t_gsw, t_conv, want_intermediates=False):
    """Full answer of one query; returns the response bytes (and optionally
    a dict with the expansion output, DB-multiply output and folded cts)."""
    lib = _load()
    g = expansion_g(nu1, nu2, t_gsw)
    T = n * n
    resp = np.zeros(response_bytes(n, pt_bits, q2_bits), dtype=np.uint8)
    exp = np.empty(((1 << g), 2, 2, D), dtype=np.uint32)
    acc = np.empty((T, 1 << nu2, 2, 2, D), dtype=np.uint32)
    folded = np.empty((T, 2, D), dtype=np.uint64)
    rc = lib.or_answer(_c(db, np.uint32), n, nu1, nu2, pt_bits, q2_bits, t_left, t_right, t_gsw,
                       t_conv, _c(query, np.uint32), _c(left, np.uint32), _c(right, np.uint32),
                       _c(conv, np.uint32), _c(pack_keys, np.uint32), resp, exp, acc, folded)
    if rc != 0:
        raise MemoryError("oracle answer: allocation failed")
    if want_intermediates:
        return resp, {"expanded": exp, "acc": acc, "folded": folded}
    return resp
