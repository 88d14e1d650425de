"""Generates the golden fixtures in this directory.

Run in a container that has scipy and the `cryptography` package:
    python tests/golden/make_golden.py

Fixtures (small, committed):
  sobol_scipy.npz   scipy.stats.qmc.Sobol(bits=32, scramble=False) points as
                    uint32 (the same Joe-Kuo D6 table and Gray-code order the
                    sobol crate uses): points 0..255 x 64 dims, and points
                    1000000..1000063 x 8 dims (fast_forward).
  chacha.json       ChaCha20 keystream blocks from `cryptography` (the ChaCha
                    core at 20 rounds, zero nonce) and the published ChaCha8
                    zero-key / zero-IV block (draft-strombergson-chacha-test-
                    vectors, TC1, 8 rounds, 256-bit key).
  icdf.json         AS 26.2.23 values computed here with the math module, an
                    independent restatement of src/proc/increment.rs:161-179.
"""
from __future__ import annotations

import json
import math
import os
import struct

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def sobol():
    from scipy.stats import qmc
    s = qmc.Sobol(d=64, scramble=False, bits=32)
    a = (s.random(256) * 2.0 ** 32).astype(np.uint64).astype(np.uint32)
    s2 = qmc.Sobol(d=8, scramble=False, bits=32)
    s2.fast_forward(1000000)
    b = (s2.random(64) * 2.0 ** 32).astype(np.uint64).astype(np.uint32)
    np.savez_compressed(os.path.join(HERE, "sobol_scipy.npz"), first256_d64=a, at1e6_d8=b)


def chacha():
    from cryptography.hazmat.primitives.ciphers import Cipher, algorithms
    out = {"chacha20": [], "chacha8_tc1": {}}
    cases = [(bytes(32), 0), (bytes(range(32)), 0), (bytes(range(32)), 7)]
    for key, counter in cases:
        nonce = struct.pack("<I", counter) + bytes(12)
        enc = Cipher(algorithms.ChaCha20(key, nonce), mode=None).encryptor()
        ks = enc.update(bytes(128))
        out["chacha20"].append({
            "key_words": list(struct.unpack("<8I", key)),
            "counter": counter,
            "blocks": [list(struct.unpack("<16I", ks[i:i + 64])) for i in (0, 64)],
        })
    # draft-strombergson-chacha-test-vectors-01, TC1, ChaCha8, 256-bit zero
    # key, zero IV: first keystream block.
    tc1 = bytes.fromhex(
        "3e00ef2f895f40d67f5bb8e81f09a5a12c840ec3ce9a7f3b181be188ef711a1e"
        "984ce172b9216f419f445367456d5619314a42a3da86b001387bfdb80e0cfe42")
    out["chacha8_tc1"] = {"key_words": [0] * 8, "counter": 0,
                          "block": list(struct.unpack("<16I", tc1))}
    with open(os.path.join(HERE, "chacha.json"), "w") as f:
        json.dump(out, f, indent=1)


def icdf():
    def as26(p):
        t = math.sqrt(-2.0 * math.log(p)) if p < 0.5 else math.sqrt(-2.0 * math.log(1.0 - p))
        c0, c1, c2 = 2.515517, 0.802853, 0.010328
        d1, d2, d3 = 1.432788, 0.189269, 0.001308
        x = t - ((c2 * t + c1) * t + c0) / (((d3 * t + d2) * t + d1) * t + 1.0)
        return -x if p < 0.5 else x
    ps = [2.0 ** -53, 1e-12, 1e-6, 0.001, 0.02425, 0.1, 0.25, 0.4999999, 0.5, 0.5000001,
          0.75, 0.9, 0.97575, 0.999, 1 - 1e-9, 1 - 2.0 ** -53]
    with open(os.path.join(HERE, "icdf.json"), "w") as f:
        json.dump({"p": ps, "x": [as26(p) for p in ps]}, f, indent=1)


if __name__ == "__main__":
    sobol()
    chacha()
    icdf()
    print("fixtures written to", HERE)
