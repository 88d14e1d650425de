"""The kernels' ChaCha8 (csrc/device/sde_chacha.h), compiled here as plain C
with the host compiler: the PCG32 key expansion and the block against the
oracle's ChaCha core (pinned to the published ChaCha8 vector), including
counters whose high word is not 0.  The header is the one the sm_103a
kernels include."""
import ctypes as C
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

HEADER_DIR = os.path.join(ROOT, "sde-sim-rs_gb300", "csrc", "device")
SHIM = r"""
#include "sde_args.h"
#include "sde_chacha.h"
void seed(unsigned long long s, sde_u32* k) { sde_seed_from_u64(s, k); }
void block(const sde_u32* k, unsigned long long ctr, sde_u32* o) { sde_chacha8_block(k, ctr, o); }
"""

COUNTERS = [0, 1, 2, 7, 1000, 2**31, 2**32 - 1, 2**32, 2**32 + 5, 2**40 + 3, 2**63 + 7, 2**64 - 1]


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("chacha")
    src = d / "shim.c"
    src.write_text(SHIM)
    so = d / "shim.so"
    subprocess.run([cc, "-O2", "-fPIC", "-shared", "-I", HEADER_DIR, str(src), "-o", str(so)], check=True)
    L = C.CDLL(str(so))
    L.seed.argtypes = [C.c_uint64, C.c_void_p]
    L.block.argtypes = [C.c_void_p, C.c_uint64, C.c_void_p]
    return L


def _blk(lib, key, ctr):
    k = np.ascontiguousarray(key, dtype=np.uint32)
    o = np.zeros(16, dtype=np.uint32)
    lib.block(k.ctypes.data, ctr, o.ctypes.data)
    return o


def test_published_chacha8_vector(lib):
    with open(os.path.join(GOLDEN, "chacha.json")) as f:
        tc1 = json.load(f)["chacha8_tc1"]
    assert _blk(lib, tc1["key_words"], tc1["counter"]).tolist() == tc1["block"]


def test_seed_expansion_matches_oracle(lib, oracle):
    for s in [0, 1, 42, 2**32 + 17, 2**64 - 1]:
        k = np.zeros(8, dtype=np.uint32)
        lib.seed(s, k.ctypes.data)
        assert np.array_equal(k, oracle.seed_from_u64(s)), s


def test_blocks_match_oracle(lib, oracle):
    rng = np.random.default_rng(7)
    keys = [oracle.seed_from_u64(s) for s in (0, 5, 123456789)]
    keys += [rng.integers(0, 2**32, 8, dtype=np.uint64).astype(np.uint32) for _ in range(5)]
    keys.append(np.full(8, 0xffffffff, dtype=np.uint32))
    for key in keys:
        for ctr in COUNTERS + [int(c) for c in rng.integers(0, 2**63, 8, dtype=np.uint64)]:
            assert np.array_equal(_blk(lib, key, ctr), oracle.chacha_block(key, ctr, 0, rounds=8)), (key, ctr)


def test_stream_u64_order(lib, oracle):
    # u64 k of the scenario's stream = words 2k (low) and 2k+1 (high) of
    # block k // 8, as the kernels pair them
    k = np.zeros(8, dtype=np.uint32)
    lib.seed(99, k.ctypes.data)
    words = np.concatenate([_blk(lib, k, b) for b in range(4)]).astype(np.uint64)
    assert np.array_equal(words[0::2] | (words[1::2] << np.uint64(32)), oracle.chacha8_u64(99, 0, 32))
