"""Known-answer vectors for the ChaCha20 block function used by the seed
expansion of public parameters (spiralpir/prg.py, csrc/seeded.cu).

    python tests/golden/make_chacha_vectors.py

Writes tests/golden/chacha20.json: for a few (key, counter, nonce) triples,
the 64-byte keystream block computed by an independent implementation (the
`cryptography` package's ChaCha20, RFC 8439), including the block-function
example of RFC 8439 section 2.3.2 (key 00..1f, counter 1, nonce
000000090000004a00000000).
"""
import json
import os

from cryptography.hazmat.primitives.ciphers import Cipher, algorithms

HERE = os.path.dirname(os.path.abspath(__file__))


def block(key: bytes, counter: int, nonce: bytes) -> bytes:
    c = Cipher(algorithms.ChaCha20(key, counter.to_bytes(4, "little") + nonce), mode=None).encryptor()
    return c.update(bytes(64))


def main() -> None:
    cases = [
        (bytes(range(32)), 1, bytes.fromhex("000000090000004a00000000")),
        (bytes(32), 0, bytes(12)),
        (bytes(range(100, 132)), 255, (7).to_bytes(4, "little") + (1).to_bytes(4, "little")
         + (0x3153504B).to_bytes(4, "little")),
        (bytes(b ^ 0xA5 for b in range(32)), 0xFFFFFFFF, bytes.fromhex("0102030405060708090a0b0c")),
    ]
    out = [{"key": k.hex(), "counter": c, "nonce": n.hex(), "block": block(k, c, n).hex()} for k, c, n in cases]
    with open(os.path.join(HERE, "chacha20.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
