"""Run the reference's own Python CPU model (gpu-pir/cpu_version) on given
inputs, in a separate process.

Usage: python ref_cpu_version.py <cpu_version dir> <work dir>

Reads <work dir>/in.npz and writes <work dir>/out.npz.  Inputs:
  ntt_in   uint32 (k, 2, D)  canonical residues; output ntt_out (k, 2, D)
           = the reference's gpu_ntt_256 per prime (cpu_version/ntt.py:201-216)
  intt_in  uint32 (k, 2, D); output intt_out = gpu_intt_256 with scaling
           (cpu_version/ntt.py:319-336)
  fold_in  uint64 (4, 2, D) raw, fold_keys / fold_keys_neg uint64
           (2, 2, 16, 2, D) in the golden-vector file layout; output fold_out
           uint64 (2, D) = fold_all_ciphertexts (cpu_version/folding.py:45-50)
Every output also gets its wall time in seconds (`<name>_s`, one core: the
model is pure Python), the reference's own CPU timing of these stages.
The reference code is used exactly as shipped (its fixture parameters
V2 = 2, T_GSW = 8); it reads its inputs through its own loaders
(cpu_version/testing.py:61-114) from files written here in the golden-vector
format.  No bytecode is written into the reference tree.
"""
import contextlib
import io
import os
import sys
import time

sys.dont_write_bytecode = True


def main(ref_dir: str, work: str) -> None:
    import numpy as np

    sys.path.insert(0, ref_dir)
    with contextlib.redirect_stdout(io.StringIO()):
        import folding  # noqa: E402  (reference module)
        import ntt as rntt  # noqa: E402
        import params as rparams  # noqa: E402
        import testing  # noqa: E402

    inp = np.load(os.path.join(work, "in.npz"))
    out = {}
    primes = [(rparams.Q1, rparams.Q1_MONT, rntt.q1_twiddles, rntt.q1_inv_twiddles),
              (rparams.Q2, rparams.Q2_MONT, rntt.q2_twiddles, rntt.q2_inv_twiddles)]
    if "ntt_in" in inp:
        t0 = time.perf_counter()
        a = inp["ntt_in"]
        res = np.empty_like(a)
        for i in range(a.shape[0]):
            for k, (q, qm, tw, _) in enumerate(primes):
                res[i, k] = rntt.gpu_ntt_256([int(x) for x in a[i, k]], q, qm, tw, True)
        out["ntt_out"] = res
        out["ntt_out_s"] = time.perf_counter() - t0
    if "intt_in" in inp:
        t0 = time.perf_counter()
        a = inp["intt_in"]
        res = np.empty_like(a)
        for i in range(a.shape[0]):
            for k, (q, qm, _, itw) in enumerate(primes):
                res[i, k] = rntt.gpu_intt_256([int(x) for x in a[i, k]], q, qm, itw, True)
        out["intt_out"] = res
        out["intt_out_s"] = time.perf_counter() - t0
    if "fold_in" in inp:
        fin = os.path.join(work, "fold_in.dat")
        fk = os.path.join(work, "fold_keys.dat")
        fkn = os.path.join(work, "fold_keys_neg.dat")
        inp["fold_in"].astype("<u8").tofile(fin)
        inp["fold_keys"].astype("<u8").tofile(fk)
        inp["fold_keys_neg"].astype("<u8").tofile(fkn)
        t = rparams.T_GSW
        with contextlib.redirect_stdout(io.StringIO()):
            cts = testing.load_polys(fin, False)
            keys = testing.load_polys(fk, True, 2 * t, True, True, True)
            keys_neg = testing.load_polys(fkn, True, 2 * t, True, True, True)
            t0 = time.perf_counter()
            folding.fold_all_ciphertexts(cts, keys, keys_neg)
            out["fold_out_s"] = time.perf_counter() - t0
        ct = cts[0]
        res = np.empty((2, len(ct.a.crt_0.data)), dtype=np.uint64)
        for r, poly in enumerate((ct.a, ct.as_e)):
            res[r] = [(h << 32) + l for h, l in zip(poly.crt_0.data, poly.crt_1.data)]
        out["fold_out"] = res
    np.savez(os.path.join(work, "out.npz"), **out)


if __name__ == "__main__":
    main(sys.argv[1], sys.argv[2])
