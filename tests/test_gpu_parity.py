"""GPU parity: every stage of the CUDA library, called through the C ABI,
against the CPU oracle on the same seeded inputs and against the committed
golden digests (bit-exact: all arithmetic is modular integer arithmetic)."""
import json
import os

import numpy as np
import pytest

import oracle as O
from golden import cases, seeded
from spiralpir import client as C
from spiralpir import params as P
from spiralpir.client import PublicKeys
from spiralpir.lib import SpiralError, SpiralGPU

pytestmark = pytest.mark.gpu

D = 2048
GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))


def digest(a):
    return cases.digest(a)


def _p(**kw):
    return P.SpiralParams(**{**dict(n=2, pt_bits=8, t_exp_left=8, t_exp_right=8, t_gsw=7, t_conv=4,
                                    q2_bits=22), **kw})


@pytest.fixture(scope="module")
def gpu():
    ctx = SpiralGPU(_p(), max_batch=8)
    yield ctx
    ctx.close()


@pytest.fixture(scope="module")
def gpu_fix():
    ctx = SpiralGPU(P.FIXTURE_PARAMS, max_batch=2)
    yield ctx
    ctx.close()


def _keys_from(left, right, conv, pack):
    return PublicKeys(exp_left=left, exp_right=right, conv=conv, pack=pack)


def test_ntt_forward(gpu):
    x = cases.inputs("ntt")
    got = gpu.ntt_fwd(x["raw"]).astype(np.uint32)
    assert np.array_equal(got, O.to_ntt(x["raw"]))
    assert digest(got) == GOLDEN["ntt"]["ntt"]


def test_ntt_inverse(gpu):
    x = cases.inputs("intt")
    got = gpu.ntt_inv(x["ntt"])
    assert np.array_equal(got, O.from_ntt(x["ntt"]))
    assert digest(got) == GOLDEN["intt"]["raw"]


def test_ntt_edge_values(gpu):
    raw = np.zeros((4, D), dtype=np.uint64)
    raw[1] = O.Q - 1                      # all q-1
    raw[2, ::2] = O.Q - 1
    raw[3] = np.arange(D, dtype=np.uint64) * np.uint64(0x0123456789)  % np.uint64(O.Q)
    got = gpu.ntt_fwd(raw).astype(np.uint32)
    assert np.array_equal(got, O.to_ntt(raw))
    assert np.array_equal(gpu.ntt_inv(got), raw)


def test_automorph(gpu):
    x = cases.inputs("automorph")
    for t in x["ts"]:
        got = gpu.automorph(x["raw"][None], t)[0]
        assert digest(got) == GOLDEN["automorph"][f"t{t}"]


def test_expansion_fixture_shape(gpu_fix):
    """Full coefficient expansion at the golden-vector parameters (t = 8,
    nu1 = 6, nu2 = 2): the selectors and GSW-bit encodings it produces."""
    x = cases.inputs("expand")
    keys = _keys_from(x["left"], x["right"], seeded.residues(9, (2, 8)), seeded.residues(10, (1, 2, 4)))
    gpu_fix.set_client_keys(1, keys)
    got = gpu_fix.expand(1, x["query"], x["nu1"], x["nu2"]).astype(np.uint32)
    ref = O.expand(x["query"], x["left"], 8, x["right"], 8, x["nu1"], x["nu2"], x["t_gsw"])
    used = [2 * k for k in range(1 << x["nu1"])] + [2 * k + 1 for k in range(x["t_gsw"] * x["nu2"])]
    assert np.array_equal(got[used], ref[used])


def test_expansion_one_round(gpu_fix):
    x = cases.inputs("expand")
    keys = _keys_from(x["left"], x["right"], seeded.residues(9, (2, 8)), seeded.residues(10, (1, 2, 4)))
    gpu_fix.set_client_keys(2, keys)
    got = gpu_fix.expand(2, x["query"], x["nu1"], x["nu2"], rounds=1).astype(np.uint32)
    ref = O.expand(x["query"], x["left"], 8, x["right"], 8, x["nu1"], x["nu2"], x["t_gsw"], rounds=1)
    assert np.array_equal(got, ref)


def test_expansion_config_shape(gpu):
    """t_gsw = 7, nu1 = 7, nu2 = 3 (g = 8, stop_round = 5): pruning and the
    left/right key rule at a shape where they matter."""
    left = seeded.residues(501, (8, 2, 8))
    right = seeded.residues(502, (6, 2, 8))
    q = seeded.residues(503, (2,))
    gpu.set_client_keys(3, _keys_from(left, right, seeded.residues(504, (2, 8)), seeded.residues(505, (2, 3, 4))))
    got = gpu.expand(3, q, 7, 3).astype(np.uint32)
    ref = O.expand(q, left, 8, right, 8, 7, 3, 7)
    used = [2 * k for k in range(128)] + [2 * k + 1 for k in range(21)]
    assert np.array_equal(got[used], ref[used])


def test_regev_to_gsw_and_neg(gpu):
    x = cases.inputs("regev_to_gsw")
    gpu.set_client_keys(4, _keys_from(seeded.residues(1, (8, 2, 8)), seeded.residues(2, (6, 2, 8)), x["conv"],
                                      seeded.residues(3, (2, 3, 4))))
    gsw = gpu.regev_to_gsw(4, x["regev"], x["nu2"]).astype(np.uint32)
    assert digest(gsw) == GOLDEN["regev_to_gsw"]["gsw"]
    assert np.array_equal(gsw, O.regev_to_gsw(x["regev"], x["conv"], x["nu2"], x["t_gsw"], x["t_conv"]))
    neg = gpu.gsw_neg(gsw).astype(np.uint32)
    assert digest(neg) == GOLDEN["regev_to_gsw"]["neg"]


def test_db_mul(gpu):
    x = cases.inputs("db_mul")
    gpu.load_db_ntt(7, x["db"], x["nu1"], x["nu2"])
    got = gpu.db_mul(7, x["sel"], x["T"], x["nu2"]).astype(np.uint32)
    assert digest(got) == GOLDEN["db_mul"]["acc"]
    gpu.unload_db(7)


def test_db_mul_extreme_values(gpu):
    """All-(q-1) selectors and database: the 64-bit accumulators run at their
    bound for 512 rows."""
    T, nu1, nu2 = 4, 9, 2
    db = np.empty((T, 1 << nu2, 1 << nu1, 2, D), dtype=np.uint32)
    db[..., 0, :] = O.Q1 - 1
    db[..., 1, :] = O.Q2 - 1
    sel = np.empty((1 << nu1, 2, 2, D), dtype=np.uint32)
    sel[..., 0, :] = O.Q1 - 1
    sel[..., 1, :] = O.Q2 - 1
    gpu.load_db_ntt(8, db, nu1, nu2)
    got = gpu.db_mul(8, sel, T, nu2).astype(np.uint32)
    assert np.array_equal(got, O.db_mul(db, sel, T, nu1, nu2))
    gpu.unload_db(8)


def _extreme_planes(shape, p, rng):
    """uint32 residues mod p mixing the digit-decomposition edge cases
    (0, 1, (p-1)/2, (p+1)/2, p-1) with uniform values."""
    edge = np.array([0, 1, (p - 1) // 2, (p + 1) // 2, p - 1], dtype=np.uint32)
    x = rng.integers(0, p, size=shape, dtype=np.uint32)
    pick = rng.integers(0, 8, size=shape)
    sel = pick < 5
    x[sel] = edge[pick[sel]]
    return x


@pytest.mark.parametrize("variant", [1, 2, 3])
def test_db_mul_batch_variants_extreme(gpu, variant):
    """512 rows (the exactness bound of the tensor-core digit products) with
    edge-case residues in the database and the selectors: every multiply
    variant equals the oracle."""
    T, nu1, nu2, nq = 4, 9, 5, 3
    rng = np.random.default_rng(11)
    db = np.empty((T, 1 << nu2, 1 << nu1, 2, D), dtype=np.uint32)
    db[..., 0, :] = _extreme_planes(db[..., 0, :].shape, O.Q1, rng)
    db[..., 1, :] = _extreme_planes(db[..., 1, :].shape, O.Q2, rng)
    sels = np.empty((nq, 1 << nu1, 2, 2, D), dtype=np.uint32)
    sels[..., 0, :] = _extreme_planes(sels[..., 0, :].shape, O.Q1, rng)
    sels[..., 1, :] = _extreme_planes(sels[..., 1, :].shape, O.Q2, rng)
    sels[0, :, :, 0, :] = (O.Q1 - 1) // 2       # all-extreme selector against the edge-heavy image
    sels[0, :, :, 1, :] = (O.Q2 + 1) // 2
    gpu.load_db_ntt(9, db, nu1, nu2)
    try:
        gpu.set_db_mul_variant(variant)
        gpu.stats_reset()
        got = gpu.db_mul_batch(9, sels, T, nu2).astype(np.uint32)
        assert gpu.stats()["db_mul_by_variant"][variant - 1] == 1
    finally:
        gpu.set_db_mul_variant(0)
        gpu.unload_db(9)
    for q in range(nq):
        assert np.array_equal(got[q], O.db_mul(db, sels[q], T, nu1, nu2)), f"query {q}"


def test_db_mul_tc_two_passes(gpu):
    """40 queries: the tensor-core multiply runs passes of 32 and 8 queries
    (N = 64 and N = 16); every output equals the per-query kernel's."""
    T, nu1, nu2, nq = 4, 7, 5, 40
    rng = np.random.default_rng(12)
    db = np.empty((T, 1 << nu2, 1 << nu1, 2, D), dtype=np.uint32)
    db[..., 0, :] = rng.integers(0, O.Q1, size=db[..., 0, :].shape, dtype=np.uint32)
    db[..., 1, :] = rng.integers(0, O.Q2, size=db[..., 1, :].shape, dtype=np.uint32)
    sels = np.empty((nq, 1 << nu1, 2, 2, D), dtype=np.uint32)
    sels[..., 0, :] = rng.integers(0, O.Q1, size=sels[..., 0, :].shape, dtype=np.uint32)
    sels[..., 1, :] = rng.integers(0, O.Q2, size=sels[..., 1, :].shape, dtype=np.uint32)
    gpu.load_db_ntt(9, db, nu1, nu2)
    try:
        gpu.set_db_mul_variant(3)
        tc = gpu.db_mul_batch(9, sels, T, nu2)
        gpu.set_db_mul_variant(1)
        ref = gpu.db_mul_batch(9, sels, T, nu2)
    finally:
        gpu.set_db_mul_variant(0)
        gpu.unload_db(9)
    assert np.array_equal(tc, ref)
    assert np.array_equal(ref[39].astype(np.uint32), O.db_mul(db, sels[39], T, nu1, nu2))


def test_db_mul_tc_n48_matches_integer_kernels(gpu):
    """24 queries: one tensor-core pass at N = 48 (selector columns padded to
    a multiple of 16); equal to the per-query and the integer batch kernels."""
    T, nu1, nu2, nq = 4, 7, 5, 24
    rng = np.random.default_rng(13)
    db = np.empty((T, 1 << nu2, 1 << nu1, 2, D), dtype=np.uint32)
    db[..., 0, :] = rng.integers(0, O.Q1, size=db[..., 0, :].shape, dtype=np.uint32)
    db[..., 1, :] = rng.integers(0, O.Q2, size=db[..., 1, :].shape, dtype=np.uint32)
    sels = np.empty((nq, 1 << nu1, 2, 2, D), dtype=np.uint32)
    sels[..., 0, :] = rng.integers(0, O.Q1, size=sels[..., 0, :].shape, dtype=np.uint32)
    sels[..., 1, :] = rng.integers(0, O.Q2, size=sels[..., 1, :].shape, dtype=np.uint32)
    gpu.load_db_ntt(9, db, nu1, nu2)
    outs = {}
    try:
        for v in (1, 2, 3):
            gpu.set_db_mul_variant(v)
            outs[v] = gpu.db_mul_batch(9, sels, T, nu2)
    finally:
        gpu.set_db_mul_variant(0)
        gpu.unload_db(9)
    assert np.array_equal(outs[3], outs[1]) and np.array_equal(outs[2], outs[1])
    assert np.array_equal(outs[3][5].astype(np.uint32), O.db_mul(db, sels[5], T, nu1, nu2))


@pytest.mark.parametrize("nu1, nu2", [(6, 2), (5, 1), (5, 3)])
def test_db_mul_batch_small_image(gpu_fix, nu1, nu2):
    """n = 1, 2 to 8 combos per block (no tensor-core shape; a packed row
    narrower than 8 combos is padded): the integer batch kernel and the
    per-query kernel equal the oracle for every query."""
    T, nq = 1, 5
    rng = np.random.default_rng(14)
    db = np.empty((T, 1 << nu2, 1 << nu1, 2, D), dtype=np.uint32)
    db[..., 0, :] = _extreme_planes(db[..., 0, :].shape, O.Q1, rng)
    db[..., 1, :] = _extreme_planes(db[..., 1, :].shape, O.Q2, rng)
    sels = np.empty((nq, 1 << nu1, 2, 2, D), dtype=np.uint32)
    sels[..., 0, :] = _extreme_planes(sels[..., 0, :].shape, O.Q1, rng)
    sels[..., 1, :] = _extreme_planes(sels[..., 1, :].shape, O.Q2, rng)
    gpu_fix.load_db_ntt(3, db, nu1, nu2)
    try:
        for v in (1, 2):
            gpu_fix.set_db_mul_variant(v)
            got = gpu_fix.db_mul_batch(3, sels, T, nu2).astype(np.uint32)
            for q in range(nq):
                assert np.array_equal(got[q], O.db_mul(db, sels[q], T, nu1, nu2)), (v, q)
    finally:
        gpu_fix.set_db_mul_variant(0)
        gpu_fix.unload_db(3)


def test_fold(gpu):
    x = cases.inputs("fold")
    got = gpu.fold(x["cts"], x["V"], x["nu2"])
    assert digest(got) == GOLDEN["fold"]["folded"]


@pytest.mark.parametrize("pattern", ["v0_max", "v1_max", "all_max"])
def test_fold_extreme_digits_match_oracle(gpu, pattern):
    """Fold inputs whose gadget digits take extreme values: the first or the
    second half of the columns (the two inputs of every level-0 fold) at
    q - 1, the others 0, so the one-product fold's digit differences reach
    both ends of [0, p) and its lazy digit transforms their largest inputs;
    the result equals the oracle's two-product fold."""
    T, nu2, t = 2, 3, 7
    half = 1 << (nu2 - 1)
    cts = np.zeros((T, 1 << nu2, 2, P.D), dtype=np.uint64)
    if pattern in ("v0_max", "all_max"):
        cts[:, :half] = P.Q - 1
    if pattern in ("v1_max", "all_max"):
        cts[:, half:] = P.Q - 1
    V = seeded.residues(131, (nu2, 2, 2 * t))
    got = gpu.fold(cts, V, nu2)
    want = O.fold(cts, V, O.gsw_neg(V, t), nu2, t)
    assert np.array_equal(got, want)


def test_pack(gpu):
    x = cases.inputs("pack")
    gpu.set_client_keys(5, _keys_from(seeded.residues(1, (8, 2, 8)), seeded.residues(2, (6, 2, 8)),
                                      seeded.residues(3, (2, 8)), x["keys"]))
    resp = gpu.pack(5, x["cts"])
    assert digest(resp) == GOLDEN["pack"]["response"]


@pytest.mark.parametrize("n,t_conv,pt_bits,q2_bits", [(1, 3, 4, 6), (2, 8, 8, 32), (4, 4, 8, 22)])
def test_pack_across_n_matches_oracle(n, t_conv, pt_bits, q2_bits):
    """The pack stage entry runs the batch pack kernel (one CTA group per
    column, n + 1 accumulators in registers, serialisation by the CTA that
    finishes each polynomial): response bytes equal the oracle's pack and
    serialisation for n = 1, 2 and 4 and the extreme first-row widths.  The
    row-per-CTA kernel that single queries use is covered at these n by
    whole answers (test_gpu_param_sets.py)."""
    p = _p(n=n, t_conv=t_conv, pt_bits=pt_bits, q2_bits=q2_bits)
    cts = seeded.raw(130 + n, (n * n, 2))
    keys = seeded.residues(140 + n, (n, n + 1, t_conv))
    with SpiralGPU(p, max_batch=1) as g:
        g.set_client_keys(1, _keys_from(seeded.residues(1, (8, 2, 8)), seeded.residues(2, (6, 2, 8)),
                                        seeded.residues(3, (2, 2 * t_conv)), keys))
        resp = g.pack(1, cts)
    ref = O.encode_response(O.pack(cts, keys, n, t_conv), n, pt_bits, q2_bits)
    assert np.array_equal(resp, ref)


def test_answer_matches_oracle(gpu):
    """The whole pipeline on seeded (non-encrypted) inputs: response bytes are
    identical to the oracle's."""
    x = cases.inputs("answer")
    gpu.set_client_keys(6, _keys_from(x["left"], x["right"], x["conv"], x["pack"]))
    gpu.load_db(9, x["records"], x["nu1"], x["nu2"])
    resp = gpu.answer(6, 9, x["query"])
    assert digest(resp) == GOLDEN["answer"]["response"]


def test_db_encode_matches_oracle(gpu):
    x = cases.inputs("answer")
    db_or = O.db_encode(x["records"], 2, x["nu1"], x["nu2"], 8)
    gpu.load_db(10, x["records"], x["nu1"], x["nu2"])
    # probe the encoded image through the multiply with unit selectors
    for row in (0, 77):
        sel = np.zeros((1 << x["nu1"], 2, 2, D), dtype=np.uint32)
        sel[row, 0] = 1
        got = gpu.db_mul(10, sel, 4, x["nu2"]).astype(np.uint32)
        assert np.array_equal(got[:, :, 0], db_or[:, :, row])
    gpu.unload_db(10)


@pytest.fixture(scope="module")
def real_client():
    p = _p()
    cl = C.Client(p, seed=21)
    keys = cl.public_keys(8, 5)
    return cl, keys


@pytest.mark.parametrize("index", [0, 1, 513, 1023])
def test_end_to_end_decode(gpu, real_client, index):
    """A real client's query answered on the GPU decodes to the record, and the
    response equals the oracle's byte for byte."""
    cl, keys = real_client
    sh = P.SHAPE_8MIB
    recs = C.random_records(sh, cl.params, seed=22)
    gpu.set_client_keys(20, keys)
    gpu.load_db(20, recs, sh.nu1, sh.nu2)
    q = cl.query(sh, index)
    resp = gpu.answer(20, 20, q)
    assert np.array_equal(cl.decode(resp), recs[index])
    db = O.db_encode(recs, 2, sh.nu1, sh.nu2, 8)
    ref = O.answer(db, q, keys.exp_left, keys.exp_right, keys.conv, keys.pack, n=2, nu1=sh.nu1, nu2=sh.nu2,
                   pt_bits=8, q2_bits=22, t_left=8, t_right=8, t_gsw=7, t_conv=4)
    assert np.array_equal(resp, ref)


def test_batch_mixed_databases_match_single(gpu, real_client):
    """Queries against two databases of different shapes answered in one batch
    give the same bytes as each answered alone."""
    cl, keys = real_client
    a, b = P.SHAPE_8MIB, P.DbShape(6, 4)
    ra = C.random_records(a, cl.params, seed=31)
    rb = C.random_records(b, cl.params, seed=32)
    gpu.set_client_keys(30, keys)
    gpu.load_db(31, ra, a.nu1, a.nu2)
    gpu.load_db(32, rb, b.nu1, b.nu2)
    reqs = [(30, 31, cl.query(a, 5)), (30, 32, cl.query(b, 700)), (30, 31, cl.query(a, 900)),
            (30, 32, cl.query(b, 3))]
    alone = [gpu.answer(c, d, q) for c, d, q in reqs]
    batch = gpu.answer_batch(reqs)
    for x, y in zip(alone, batch):
        assert np.array_equal(x, y)
    assert np.array_equal(cl.decode(batch[1]), rb[700])
    assert np.array_equal(cl.decode(batch[2]), ra[900])


def test_staged_answer_matches(gpu, real_client):
    cl, keys = real_client
    sh = P.SHAPE_8MIB
    recs = C.random_records(sh, cl.params, seed=41)
    gpu.set_client_keys(40, keys)
    gpu.load_db(40, recs, sh.nu1, sh.nu2)
    q = cl.query(sh, 321)
    gpu.stage_query(0, 40, 40, q)
    gpu.run_staged(1)
    gpu.run_staged(1)      # the staged query survives repeated runs
    r1 = gpu.fetch_response(0)
    assert gpu.time_db_mul(40, 1, 3) > 0
    assert gpu.time_staged(1, 2) > 0
    assert np.array_equal(gpu.fetch_response(0), r1)
    assert np.array_equal(r1, gpu.answer(40, 40, q))   # answering reuses the slots
    assert np.array_equal(cl.decode(r1), recs[321])
    with pytest.raises(SpiralError):
        gpu.run_staged(1)                                # staged queries were consumed


def test_fixture_params_end_to_end(gpu_fix):
    """n = 1 with the golden-vector gadgets (t_gsw = 8) and shape (6, 2)."""
    p = P.FIXTURE_PARAMS
    cl = C.Client(p, seed=51)
    keys = cl.public_keys(6, 2)
    sh = P.FIXTURE_SHAPE
    recs = C.random_records(sh, p, seed=52)
    gpu_fix.set_client_keys(50, keys)
    gpu_fix.load_db(50, recs, sh.nu1, sh.nu2)
    for idx in (0, 100, 255):
        resp = gpu_fix.answer(50, 50, cl.query(sh, idx))
        assert np.array_equal(cl.decode(resp), recs[idx])


def test_errors_are_reported(gpu):
    q = np.zeros((2, 2, D), dtype=np.uint64)
    with pytest.raises(SpiralError) as e:
        gpu.answer(12345, 20, q)
    assert e.value.code == 4
    with pytest.raises(SpiralError) as e:
        gpu.load_db(99, np.zeros((10, 4, D), dtype=np.uint8), 3, 3)
    assert e.value.code == 1


def test_database_unit_too_small_rejected(gpu_fix):
    """A unit of the packed image (2^nu1 rows x 8 combo places) must be at
    least 32 residue places (a whole number of 16-byte copies)."""
    with pytest.raises(SpiralError) as e:
        gpu_fix.load_db(77, np.zeros((4, 1, D), dtype=np.uint8), 1, 1)
    assert e.value.code == 6
    with pytest.raises(SpiralError):
        gpu_fix.load_db_ntt(77, np.zeros((1, 2, 2, 2, D), dtype=np.uint32), 1, 1)


def test_hbm_budget_admission():
    small = SpiralGPU(_p(), hbm_budget_bytes=64 << 20, max_batch=1)
    try:
        recs = np.zeros((1 << 11, 4, D), dtype=np.uint8)
        with pytest.raises(SpiralError) as e:
            small.load_db(1, recs, 7, 4)      # 112 MiB image does not fit the budget
        assert e.value.code == 3
    finally:
        small.close()
