"""The kernels' 32-bit form of the reference's shifted Sobol uniform
(csrc/device/sde_shift.h), compiled here as plain C with the host compiler:
U = fract(x 2^-32 + (r >> 11) 2^-53) in units of 2^-53, as the f64 sum
rounds it (src/rng/sobol.rs:62-79), bit for bit, and the tail pieces and
their float within one ulp.  The header is the one the sm_103a kernels
include."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

HEADER_DIR = os.path.join(ROOT, "sde-sim-rs_gb300", "csrc", "device")
SHIM = r"""
#include <math.h>
#include "sde_args.h"
#include "sde_shift.h"
void run(const sde_u32* x, const sde_u64* r, long n, sde_u32* hi, sde_u32* lo, sde_u32* hq, sde_u32* lq,
         int* up, float* qf) {
    for (long i = 0; i < n; ++i) {
        sde_shift_split(x[i], r[i], &hi[i], &lo[i]);
        sde_tail_split(hi[i], lo[i], &hq[i], &lq[i], &up[i]);
        qf[i] = fmaf((float)hq[i], 0x1p21f, (float)lq[i]);
    }
}
"""


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("shift")
    src = d / "shim.c"
    src.write_text(SHIM)
    so = d / "shim.so"
    subprocess.run([cc, "-O2", "-std=c11", "-ffp-contract=off", "-fPIC", "-shared", "-I", HEADER_DIR, str(src),
                    "-o", str(so), "-lm"], check=True)
    L = C.CDLL(str(so))
    L.run.argtypes = [C.c_void_p] * 2 + [C.c_long] + [C.c_void_p] * 6
    return L


def _cases():
    rng = np.random.default_rng(2025)
    n = 1 << 20
    x = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    r = rng.integers(0, 2**64 - 1, n, dtype=np.uint64, endpoint=True)
    # edges: sums at and around 1, ties (odd low bits, with and without bit
    # 1), low bits all ones (the rounding carries into bit 21), extremes
    xs, rs = [], []
    for xv in (0, 1, 2**31, 2**32 - 2, 2**32 - 1):
        for rh in (0, 1, 2**32 - 1 - xv, 2**32 - xv if xv else 0, 2**32 - 1, 2**31):
            for rl in (0, 1, 2, 3, 5, 6, 7, 2**21 - 1, 2**21 - 2, 2**21 - 3, 2**20, 2**20 + 1):
                for junk in (0, 2**11 - 1):
                    xs.append(xv)
                    rs.append(((rh % 2**32) << 32) | (rl << 11) | junk)
    x = np.concatenate([x, np.array(xs, dtype=np.uint32)])
    r = np.concatenate([r, np.array(rs, dtype=np.uint64)])
    return x, r


def test_shift_split_matches_the_f64_sum(lib):
    x, r = _cases()
    n = len(x)
    out = {k: np.zeros(n, dtype=np.uint32) for k in ("hi", "lo", "hq", "lq")}
    up = np.zeros(n, dtype=np.int32)
    qf = np.zeros(n, dtype=np.float32)
    lib.run(x.ctypes.data, r.ctypes.data, n, out["hi"].ctypes.data, out["lo"].ctypes.data, out["hq"].ctypes.data,
            out["lq"].ctypes.data, up.ctypes.data, qf.ctypes.data)
    # the reference: v = x 2^-32 + (r >> 11) 2^-53 in f64, u = v - trunc(v)
    v = x.astype(np.float64) * 2.0 ** -32 + (r >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
    u = v - np.trunc(v)
    U = (u * 2.0 ** 53).astype(np.uint64)
    assert np.all(U.astype(np.float64) * 2.0 ** -53 == u)          # u is a whole number of units
    assert np.all(out["lo"] < 2 ** 21)
    got = (out["hi"].astype(np.uint64) << np.uint64(21)) | out["lo"].astype(np.uint64)
    np.testing.assert_array_equal(got, U)
    # the tail Q = min(U, 2^53 - U), up = U >= 2^52
    Q = np.where(U >= np.uint64(2 ** 52), np.uint64(2 ** 53) - U, U)
    np.testing.assert_array_equal(up.astype(bool), U >= np.uint64(2 ** 52))
    np.testing.assert_array_equal((out["hq"].astype(np.uint64) << np.uint64(21)) | out["lq"].astype(np.uint64), Q)
    # its float within one ulp of the correctly rounded one
    exact = Q.astype(np.float32)
    ulp = np.spacing(np.abs(exact))
    assert np.all(np.abs(qf.astype(np.float64) - exact.astype(np.float64)) <= ulp.astype(np.float64))
