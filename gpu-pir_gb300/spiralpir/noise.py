"""Noise diagnostics of the answer path (host side, through the library's
stage entry points and answers).

    python -m spiralpir.noise [--nu1 9] [--nu2 11] [--t-exp-right 8 16]
                              [--clients 4] [--queries 4] [--json out.json]

For each expansion gadget of the GSW-bit branch (t_exp_right) it measures,
with the client's secret key:

* the noise of the coefficient-expansion outputs (sp_expand): first-dimension
  selectors and GSW-bit encodings, decrypted (phase = row1 + s*row0, minus
  the expected message), as the standard deviation and the largest
  coefficient, against a model of the expansion: every round doubles the
  variance (v + tau(v)) and adds the key switch's t*D*E[digit^2]*sigma^2
  (unsigned digits of b bits uniform in [0, 2^b), the top digit of
  56 - b*(t-1) bits), starting from the query's sigma^2 (sigma = 6.4);
* the decode margin of whole answers against a database of the shape
  (client.decode_margin: the largest distance, in units of the response
  rows' modulus 4p, from the exact plaintext multiple; decoding fails at
  2.0), and how many records decode.

The arithmetic of every stage is bit-exact against the CPU oracle, so the
noise measured here is the noise of the parameters, not of this
implementation.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import math

import numpy as np

from . import client as C
from . import params as P
from . import ring
from .lib import SpiralGPU


def phase(cl: C.Client, ct) -> np.ndarray:
    """Decryption phase of a Regev ciphertext (2 rows, 2, D) NTT form:
    row1 + s*row0 as centred int64 coefficients."""
    ct = np.asarray(ct, dtype=np.uint64)
    ph = ring.add(ct[1], ring.mul(cl.s_ntt, ct[0]))
    raw = ring.from_ntt(ph).astype(np.int64)
    return np.where(raw > P.Q // 2, raw - P.Q, raw)


def digit_var(t: int) -> float:
    """Mean of d^2 over the t unsigned gadget digits (b = ceil(56/t) bits,
    the top digit 56 - b(t-1) bits), digits uniform."""
    b = P.bits_per(t)
    widths = [b] * (t - 1) + [P.MOD_BITS - b * (t - 1)]
    return sum((2 ** w - 1) * (2 ** (w + 1) - 1) / 6 for w in widths) / t


def model_var(rounds_keys: list[int], sigma: float = C.SIGMA) -> float:
    """Expansion output noise variance after rounds using gadget lengths
    rounds_keys[r] (variance doubles, then the key switch adds its part)."""
    v = sigma ** 2
    for t in rounds_keys:
        v = 2 * v + t * P.D * digit_var(t) * sigma ** 2
    return v


def expansion_noise(gpu, cl: C.Client, client_id: int, sh: P.DbShape, index: int) -> dict:
    p = cl.params
    g = p.g(sh.nu1, sh.nu2)
    stop = p.stop_round(sh.nu2)
    rest = min(stop + 1, g)
    out = gpu.expand(client_id, cl.query(sh, index), sh.nu1, sh.nu2)
    row, col = divmod(index, sh.cols)
    sel, gsw = [], []
    for r in range(sh.rows):
        e = phase(cl, out[2 * r])
        e[0] -= P.delta(p) if r == row else 0
        sel.append(e)
    b = P.bits_per(p.t_gsw)
    for i in range(sh.nu2):
        for j in range(p.t_gsw):
            e = phase(cl, out[2 * (i * p.t_gsw + j) + 1])
            m = (((col >> i) & 1) << (b * j)) % P.Q
            e[0] -= m if m <= P.Q // 2 else m - P.Q
            gsw.append(e)
    sel, gsw = np.array(sel, dtype=np.float64), np.array(gsw, dtype=np.float64)
    # model: selectors take round 0 with the right keys, later rounds left;
    # the GSW bits take the right keys for `rest` rounds
    return {"sel_std": float(sel.std()), "sel_max": float(np.abs(sel).max()),
            "gsw_std": float(gsw.std()), "gsw_max": float(np.abs(gsw).max()),
            "model_sel_std": math.sqrt(model_var([p.t_exp_right] + [p.t_exp_left] * (g - 1))),
            "model_gsw_std": math.sqrt(model_var([p.t_exp_right] * rest))}


def run(nu1: int, nu2: int, t_rights: list[int], clients: int, queries: int) -> list[dict]:
    sh = P.DbShape(nu1, nu2)
    recs = C.random_records(sh, P.PARAMS, seed=901)
    rows = []
    for tr in t_rights:
        p = dataclasses.replace(P.PARAMS, t_exp_right=tr)
        rng = np.random.default_rng(902)
        with SpiralGPU(p, max_batch=1) as gpu:
            gpu.load_db(1, recs, sh.nu1, sh.nu2)
            noise, margins, ok = [], [], 0
            for k in range(clients):
                cl = C.Client(p, seed=910 + k)
                gpu.set_client_keys(k, cl.public_keys(sh.nu1, sh.nu2))
                for _ in range(queries):
                    idx = int(rng.integers(0, sh.num_records))
                    noise.append(expansion_noise(gpu, cl, k, sh, idx))
                    resp = gpu.answer(k, 1, cl.query(sh, idx))
                    margins.append(cl.decode_margin(resp, recs[idx]))
                    ok += bool(np.array_equal(cl.decode(resp), recs[idx]))
        n = len(margins)
        rows.append({"nu1": nu1, "nu2": nu2, "t_exp_left": p.t_exp_left, "t_exp_right": tr, "t_gsw": p.t_gsw,
                     "queries": n,
                     "sel_std_log2": math.log2(np.mean([x["sel_std"] for x in noise])),
                     "sel_model_std_log2": math.log2(noise[0]["model_sel_std"]),
                     "gsw_std_log2": math.log2(np.mean([x["gsw_std"] for x in noise])),
                     "gsw_model_std_log2": math.log2(noise[0]["model_gsw_std"]),
                     "gsw_max_log2": math.log2(max(x["gsw_max"] for x in noise)),
                     "margin_max": float(max(margins)), "margin_median": float(np.median(margins)),
                     "decoded": ok})
    return rows


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--nu1", type=int, default=9)
    ap.add_argument("--nu2", type=int, default=11)
    ap.add_argument("--t-exp-right", type=int, nargs="+", default=[8, 16])
    ap.add_argument("--clients", type=int, default=4)
    ap.add_argument("--queries", type=int, default=4)
    ap.add_argument("--json", default=None)
    a = ap.parse_args()
    rows = run(a.nu1, a.nu2, a.t_exp_right, a.clients, a.queries)
    print("| nu1, nu2 | t_exp_right | selector noise std (log2) measured / model | GSW-bit noise std (log2) "
          "measured / model | GSW-bit max (log2) | decode margin median / max (fails at 2.0) | decoded |")
    print("|---|---|---|---|---|---|---|")
    for r in rows:
        print(f"| {r['nu1']}, {r['nu2']} | {r['t_exp_right']} | {r['sel_std_log2']:.2f} / {r['sel_model_std_log2']:.2f} "
              f"| {r['gsw_std_log2']:.2f} / {r['gsw_model_std_log2']:.2f} | {r['gsw_max_log2']:.2f} "
              f"| {r['margin_median']:.3f} / {r['margin_max']:.3f} | {r['decoded']} of {r['queries']} |")
    if a.json:
        with open(a.json, "w") as f:
            json.dump(rows, f, indent=1)


if __name__ == "__main__":
    main()
