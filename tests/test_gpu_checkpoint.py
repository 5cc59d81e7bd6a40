"""GPU tests of the database image checkpoint (sp_db_save / sp_db_restore):
a restored image answers exactly like the encoded one, and damaged or
mismatched files are rejected without loading anything."""
import os

import numpy as np
import pytest

from spiralpir import client as C
from spiralpir import params as P
from spiralpir.lib import SpiralError, SpiralGPU

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def saved(tmp_path_factory):
    p = P.PARAMS
    sh = P.SHAPE_8MIB
    recs = C.random_records(sh, p, seed=71)
    cl = C.Client(p, seed=72)
    path = str(tmp_path_factory.mktemp("ckpt") / "db8mib.img")
    with SpiralGPU(p) as gpu:
        gpu.set_client_keys(1, cl.public_keys(sh.nu1, sh.nu2))
        gpu.load_db(1, recs, sh.nu1, sh.nu2)
        q = cl.query(sh, 321)
        ref = gpu.answer(1, 1, q)
        gpu.save_db(1, path)
    return p, sh, recs, cl, q, ref, path


def test_restore_answers_like_encoded(saved):
    """Restored image and freshly encoded database, same context and keys:
    byte-identical responses (public keys are randomised per generation, so
    responses are compared within one context)."""
    p, sh, recs, cl, q, ref, path = saved
    # 64-byte header + image: two 28-bit residues (7 bytes) per coefficient
    assert os.path.getsize(path) == 64 + sh.rows * sh.cols * p.n * p.n * P.D * 7
    with SpiralGPU(p) as gpu:
        gpu.set_client_keys(1, cl.public_keys(sh.nu1, sh.nu2))
        gpu.load_db(1, recs, sh.nu1, sh.nu2)
        gpu.restore_db(5, path)
        for i in (321, 0, sh.num_records - 1):
            qi = cl.query(sh, i)
            a, b = gpu.answer(1, 1, qi), gpu.answer(1, 5, qi)
            assert np.array_equal(a, b)
            assert np.array_equal(cl.decode(b), recs[i])


def test_damaged_or_mismatched_images_rejected(saved, tmp_path):
    p, sh, recs, cl, q, ref, path = saved
    blob = open(path, "rb").read()
    flipped = tmp_path / "flipped.img"
    b = bytearray(blob)
    b[64 + 12345] ^= 0x40
    flipped.write_bytes(bytes(b))
    short = tmp_path / "short.img"
    short.write_bytes(blob[: len(blob) // 2])
    junk = tmp_path / "junk.img"
    junk.write_bytes(b"not an image" * 10)
    with SpiralGPU(p) as gpu:
        for bad in (flipped, short, junk):
            with pytest.raises(SpiralError) as e:
                gpu.restore_db(7, str(bad))
            assert e.value.code == 1
        with pytest.raises(SpiralError) as e:
            gpu.restore_db(7, str(tmp_path / "missing.img"))
        assert e.value.code == 7
        used = gpu.hbm_used()
        gpu.restore_db(7, path)          # a good file still loads afterwards
        assert gpu.hbm_used() > used
    with SpiralGPU(P.FIXTURE_PARAMS) as other:   # n = 1 context: image is for n = 2
        with pytest.raises(SpiralError) as e:
            other.restore_db(1, path)
        assert e.value.code == 1
