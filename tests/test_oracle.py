"""CPU tests of the oracle: pinned to the reference's golden vectors and to
the reference's own Python model, checked against the committed digests,
and end-to-end (decoded record == database record)."""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np
import pytest

import oracle as O
from golden import cases, seeded
from spiralpir import client as C
from spiralpir import params as P
from spiralpir import ring

from conftest import REF_CPU

D = 2048
GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))


def _u64(ref_data, f):
    return np.fromfile(os.path.join(ref_data, f), dtype="<u8")


def test_ntt_golden_vector(ref_data):
    raw = _u64(ref_data, "raw_poly.dat")
    nt = _u64(ref_data, "ntt_poly.dat").reshape(2, D)
    mod = np.array([[O.Q1], [O.Q2]], dtype=np.uint64)
    assert np.array_equal(O.to_ntt(raw).astype(np.uint64), nt % mod)
    assert np.array_equal(O.from_ntt(O.to_ntt(raw)), raw % np.uint64(O.Q))


def test_fold_golden_vector(ref_data):
    fin = _u64(ref_data, "client_fold_input.dat").reshape(1, 4, 2, D)
    V = _u64(ref_data, "client_folding_keys.dat").reshape(2, 2, 16, 2, D).astype(np.uint32)
    Vn = _u64(ref_data, "client_folding_keys_neg.dat").reshape(2, 2, 16, 2, D).astype(np.uint32)
    out = _u64(ref_data, "client_fold_output.dat").reshape(2, D)
    assert np.array_equal(O.fold(fin, V, Vn, 2, 8)[0], out)


def test_gsw_neg_golden_vector(ref_data):
    V = _u64(ref_data, "client_folding_keys.dat").reshape(2, 2, 16, 2, D).astype(np.uint32)
    Vn = _u64(ref_data, "client_folding_keys_neg.dat").reshape(2, 2, 16, 2, D).astype(np.uint32)
    assert np.array_equal(O.gsw_neg(V, 8), Vn)


def test_expansion_round0_golden_vector(ref_data):
    q = _u64(ref_data, "client_expand_input.dat").reshape(2, 2, D).astype(np.uint32)
    L = _u64(ref_data, "client_expand_left_keys.dat").reshape(7, 2, 8, 2, D).astype(np.uint32)
    R = _u64(ref_data, "client_expand_right_keys.dat").reshape(5, 2, 8, 2, D).astype(np.uint32)
    out = _u64(ref_data, "client_expand_output_1round.dat").reshape(2, 2, 2, D)
    assert np.array_equal(O.expand(q, L, 8, R, 8, 6, 2, 8, rounds=1).astype(np.uint64), out)


@pytest.mark.slow
def test_oracle_matches_reference_python():
    """The reference's own cpu_version (run unmodified in a subprocess)
    agrees with the oracle on seeded NTT, INTT and fold inputs."""
    if not os.path.isdir(REF_CPU):
        pytest.skip("reference cpu_version not present")
    ntt_in = seeded.residues(301, (1,))
    fold_in = seeded.raw(302, (4, 2))
    keys = seeded.residues(303, (2, 2, 16))
    keys_neg = O.gsw_neg(keys, 8)
    with tempfile.TemporaryDirectory() as work:
        np.savez(os.path.join(work, "in.npz"), ntt_in=ntt_in, fold_in=fold_in,
                 fold_keys=keys.astype(np.uint64), fold_keys_neg=keys_neg.astype(np.uint64))
        script = os.path.join(os.path.dirname(__file__), "golden", "ref_cpu_version.py")
        subprocess.run([sys.executable, script, REF_CPU, work], check=True, cwd=work,
                       env=dict(os.environ, PYTHONDONTWRITEBYTECODE="1"))
        ref = np.load(os.path.join(work, "out.npz"))
    assert np.array_equal(ref["ntt_out"], O.ntt(ntt_in))
    assert np.array_equal(ref["fold_out"], O.fold(fold_in[None], keys, keys_neg, 2, 8)[0])


@pytest.mark.parametrize("name", cases.CASES)
def test_oracle_golden_digests(name):
    outs = cases.oracle_outputs(name)
    assert {k: cases.digest(v) for k, v in outs.items()} == GOLDEN[name]


def test_client_ring_matches_oracle():
    raw = seeded.raw(401, (3,))
    assert np.array_equal(ring.to_ntt(raw).astype(np.uint32), O.to_ntt(raw))
    a = seeded.residues(402, (3,))
    assert np.array_equal(ring.from_ntt(a.astype(np.uint64)), O.from_ntt(a))
    for t in (3, 2049, 1025):
        assert np.array_equal(ring.automorph(raw[0], t), O.automorph(raw[0], t))


def test_rescale_matches():
    rng = np.random.default_rng(5)
    xs = rng.integers(0, O.Q, size=200, dtype=np.uint64)
    xs[:4] = [0, 1, O.Q // 2, O.Q - 1]
    for q_out in (1 << 10, 1 << 22):
        got = ring.rescale(xs, O.Q, q_out)
        want = [O.rescale(int(x), O.Q, q_out) for x in xs]
        assert list(got) == want


def test_db_mul_identity_selector():
    """Selector = Enc-free unit vector: the multiply returns the chosen row."""
    T, nu1, nu2 = 1, 3, 2
    db = seeded.residues(403, (T, 4, 8))
    sel = np.zeros((8, 2, 2, D), dtype=np.uint32)
    sel[5, 0] = 1
    sel[5, 1] = 2
    acc = O.db_mul(db, sel, T, nu1, nu2)
    assert np.array_equal(acc[0, :, 0], db[0, :, 5])
    assert np.array_equal(acc[0, :, 1].astype(np.uint64),
                          (2 * db[0, :, 5].astype(np.uint64)) % np.array([[O.Q1], [O.Q2]], dtype=np.uint64))


@pytest.mark.parametrize("index", [0, 357, 1023])
def test_oracle_end_to_end_decode(index):
    """A real client's query answered by the oracle decodes to the record."""
    p, sh = P.PARAMS, P.SHAPE_8MIB
    cl = C.Client(p, seed=11)
    pk = cl.public_keys(sh.nu1, sh.nu2)
    recs = C.random_records(sh, p, seed=12)
    db = O.db_encode(recs, p.n, sh.nu1, sh.nu2, p.pt_bits)
    resp = O.answer(db, cl.query(sh, index), pk.exp_left, pk.exp_right, pk.conv, pk.pack,
                    n=p.n, nu1=sh.nu1, nu2=sh.nu2, pt_bits=p.pt_bits, q2_bits=p.q2_bits,
                    t_left=p.t_exp_left, t_right=p.t_exp_right, t_gsw=p.t_gsw, t_conv=p.t_conv)
    assert np.array_equal(cl.decode(resp), recs[index])


def test_oracle_detects_planted_mistake():
    """A single flipped residue in the oracle's input changes its output:
    the digests are sensitive to one-element errors."""
    x = cases.inputs("fold")
    V = x["V"].copy()
    base = O.fold(x["cts"], V, O.gsw_neg(V, 7), 3, 7)
    V[0, 0, 0, 0, 0] ^= 1
    bad = O.fold(x["cts"], V, O.gsw_neg(V, 7), 3, 7)
    assert not np.array_equal(base, bad)
