"""Golden cases: seeded inputs for every stage of the answer path.

Each case builds its inputs from the splitmix64 stream in seeded.py, so the
same arrays are produced on any machine.  `oracle_outputs(case)` runs the CPU
oracle on them; golden.json holds the sha256 of those outputs (made by
make_golden.py), and the GPU parity tests compare the CUDA library's
outputs with both the oracle and these digests.
"""
from __future__ import annotations

import hashlib

import numpy as np

import seeded

D = seeded.D

# Stage shapes (small enough for the oracle to finish in seconds).
FIX = dict(nu1=6, nu2=2, t_left=8, t_right=8, t_gsw=8, t_conv=4)     # golden-vector params
SMALL = dict(n=2, pt_bits=8, q2_bits=22, nu1=7, nu2=3, t_left=8, t_right=8, t_gsw=7, t_conv=4)


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def inputs(name: str) -> dict:
    s = seeded
    if name == "ntt":
        return {"raw": s.raw(101, (8,))}
    if name == "intt":
        return {"ntt": s.residues(102, (8,))}
    if name == "automorph":
        return {"raw": s.raw(103, (1,))[0], "ts": [3, 5, 1025, 2049, 4095]}
    if name == "expand":
        f = FIX
        g = 7  # ceil(log2(8*2 + 64))
        return {"query": s.residues(104, (2,)), "left": s.residues(105, (g, 2, f["t_left"])),
                "right": s.residues(106, (5, 2, f["t_right"])), **f}
    if name == "regev_to_gsw":
        return {"regev": s.residues(107, (3 * 7, 2)), "conv": s.residues(108, (2, 8)),
                "nu2": 3, "t_gsw": 7, "t_conv": 4}
    if name == "db_mul":
        return {"db": s.residues(109, (4, 8, 32)), "sel": s.residues(110, (32, 2)), "T": 4,
                "nu1": 5, "nu2": 3}
    if name == "fold":
        return {"cts": s.raw(111, (4, 8, 2)), "V": s.residues(112, (3, 2, 14)), "nu2": 3,
                "t_gsw": 7}
    if name == "pack":
        return {"cts": s.raw(113, (4, 2)), "keys": s.residues(114, (2, 3, 4)), "n": 2,
                "t_conv": 4, "pt_bits": 8, "q2_bits": 22}
    if name == "answer":
        c = SMALL
        g = 8  # ceil(log2(7*3 + 128))
        recs = s.bytes_(115, ((1 << (c["nu1"] + c["nu2"])), 4, D))
        return {"records": recs, "query": s.residues(116, (2,)),
                "left": s.residues(117, (g, 2, c["t_left"])),
                "right": s.residues(118, (6, 2, c["t_right"])),
                "conv": s.residues(119, (2, 2 * c["t_conv"])),
                "pack": s.residues(120, (2, 3, c["t_conv"])), **c}
    raise KeyError(name)


CASES = ["ntt", "intt", "automorph", "expand", "regev_to_gsw", "db_mul", "fold", "pack", "answer"]


def oracle_outputs(name: str) -> dict:
    """Oracle outputs of a case as a dict of arrays."""
    import oracle as O

    x = inputs(name)
    if name == "ntt":
        return {"ntt": O.to_ntt(x["raw"])}
    if name == "intt":
        return {"raw": O.from_ntt(x["ntt"])}
    if name == "automorph":
        return {f"t{t}": O.automorph(x["raw"], t) for t in x["ts"]}
    if name == "expand":
        return {"v": O.expand(x["query"], x["left"], x["t_left"], x["right"], x["t_right"],
                              x["nu1"], x["nu2"], x["t_gsw"])}
    if name == "regev_to_gsw":
        gsw = O.regev_to_gsw(x["regev"], x["conv"], x["nu2"], x["t_gsw"], x["t_conv"])
        return {"gsw": gsw, "neg": O.gsw_neg(gsw, x["t_gsw"])}
    if name == "db_mul":
        return {"acc": O.db_mul(x["db"], x["sel"], x["T"], x["nu1"], x["nu2"])}
    if name == "fold":
        return {"folded": O.fold(x["cts"], x["V"], O.gsw_neg(x["V"], x["t_gsw"]), x["nu2"],
                                 x["t_gsw"])}
    if name == "pack":
        packed = O.pack(x["cts"], x["keys"], x["n"], x["t_conv"])
        return {"packed": packed,
                "response": O.encode_response(packed, x["n"], x["pt_bits"], x["q2_bits"])}
    if name == "answer":
        db = O.db_encode(x["records"], x["n"], x["nu1"], x["nu2"], x["pt_bits"])
        resp, inter = O.answer(db, x["query"], x["left"], x["right"], x["conv"], x["pack"],
                               n=x["n"], nu1=x["nu1"], nu2=x["nu2"], pt_bits=x["pt_bits"],
                               q2_bits=x["q2_bits"], t_left=x["t_left"], t_right=x["t_right"],
                               t_gsw=x["t_gsw"], t_conv=x["t_conv"], want_intermediates=True)
        return {"db": db, "response": resp, "acc": inter["acc"], "folded": inter["folded"]}
    raise KeyError(name)
