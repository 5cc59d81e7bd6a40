"""Regenerate tests/golden/golden.json.

    python tests/golden/make_golden.py [--ref <reference checkout>/gpu-pir]

1. Pins the CPU oracle: when the reference tree is present, the oracle must
   reproduce the reference's golden vectors (gpu-pir/test_data/*.dat: NTT,
   one expansion round, fold, G - V) and the outputs of the reference's own
   Python model (cpu_version: NTT, INTT, fold) on seeded inputs.
2. Writes the sha256 digests of the oracle's outputs for every case in
   cases.py.  The digests (not the reference's data) are what is committed.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import cases  # noqa: E402
import oracle as O  # noqa: E402
import seeded  # noqa: E402

D = seeded.D


def pin_against_reference_vectors(test_data: str) -> None:
    def u64(f):
        return np.fromfile(os.path.join(test_data, f), dtype="<u8")

    raw = u64("raw_poly.dat")
    nt = u64("ntt_poly.dat").reshape(2, D)
    mod = np.array([[O.Q1], [O.Q2]], dtype=np.uint64)
    assert np.array_equal(O.to_ntt(raw).astype(np.uint64), nt % mod), "NTT golden vector"
    fin = u64("client_fold_input.dat").reshape(1, 4, 2, D)
    V = u64("client_folding_keys.dat").reshape(2, 2, 16, 2, D).astype(np.uint32)
    Vn = u64("client_folding_keys_neg.dat").reshape(2, 2, 16, 2, D).astype(np.uint32)
    assert np.array_equal(O.fold(fin, V, Vn, 2, 8)[0], u64("client_fold_output.dat").reshape(2, D))
    assert np.array_equal(O.gsw_neg(V, 8), Vn), "G - V golden vector"
    q = u64("client_expand_input.dat").reshape(2, 2, D).astype(np.uint32)
    L = u64("client_expand_left_keys.dat").reshape(7, 2, 8, 2, D).astype(np.uint32)
    R = u64("client_expand_right_keys.dat").reshape(5, 2, 8, 2, D).astype(np.uint32)
    out = u64("client_expand_output_1round.dat").reshape(2, 2, 2, D)
    assert np.array_equal(O.expand(q, L, 8, R, 8, 6, 2, 8, rounds=1).astype(np.uint64), out)
    print("oracle reproduces the reference golden vectors")


def pin_against_reference_python(cpu_dir: str) -> None:
    ntt_in = seeded.residues(201, (2,))
    intt_in = seeded.residues(202, (2,))
    fold_in = seeded.raw(203, (4, 2))
    keys = seeded.residues(204, (2, 2, 16))
    keys_neg = O.gsw_neg(keys, 8)
    with tempfile.TemporaryDirectory() as work:
        np.savez(os.path.join(work, "in.npz"), ntt_in=ntt_in, intt_in=intt_in, fold_in=fold_in,
                 fold_keys=keys.astype(np.uint64), fold_keys_neg=keys_neg.astype(np.uint64))
        env = dict(os.environ, PYTHONDONTWRITEBYTECODE="1")
        subprocess.run([sys.executable, os.path.join(HERE, "ref_cpu_version.py"), cpu_dir, work],
                       check=True, env=env, cwd=work)
        ref = np.load(os.path.join(work, "out.npz"))
        assert np.array_equal(ref["ntt_out"], O.ntt(ntt_in)), "reference NTT"
        ref_intt = ref["intt_out"].astype(np.uint64)
        mine = np.empty_like(ref_intt)
        for i in range(intt_in.shape[0]):
            for k in range(2):
                a = intt_in[i, k].copy()
                O._load().or_ntt_inv(a, k)
                mine[i, k] = a
        assert np.array_equal(ref_intt, mine), "reference INTT"
        assert np.array_equal(ref["fold_out"], O.fold(fold_in[None], keys, keys_neg, 2, 8)[0]), \
            "reference fold"
    print("oracle reproduces the reference cpu_version on seeded inputs")


def _reference_root() -> str:
    """$SPIRAL_REF_ROOT, else a `reference` directory beside the repository."""
    return os.environ.get("SPIRAL_REF_ROOT") or os.path.join(os.path.dirname(ROOT), "reference")


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.path.join(_reference_root(), "gpu-pir"))
    args = ap.parse_args()
    if os.path.isdir(os.path.join(args.ref, "test_data")):
        pin_against_reference_vectors(os.path.join(args.ref, "test_data"))
        pin_against_reference_python(os.path.join(args.ref, "cpu_version"))
    else:
        print("reference tree absent: digests are computed without re-pinning")
    golden = {}
    for name in cases.CASES:
        outs = cases.oracle_outputs(name)
        golden[name] = {k: cases.digest(v) for k, v in sorted(outs.items())}
        print(name, {k: v[:12] for k, v in golden[name].items()})
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(golden, f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main()
