"""The table-driven logarithm of the FP64 inverse CDF (csrc/device/sde_log.h),
compiled here as plain C with the host compiler (no FMA contraction), against
mpmath at 60 digits and against the C library's log (which the oracle, like
the reference, calls).  The header is the one the sm_103a kernels include."""
import ctypes as C
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

HEADER_DIR = os.path.join(ROOT, "sde-sim-rs_gb300", "csrc", "device")
SHIM = r"""
#include "sde_log.h"
void log_tail_batch(const double* x, double* y, long n) {
    for (long i = 0; i < n; ++i) y[i] = sde_log_tail(x[i]);
}
double as26(double p) {  /* the FP64 inverse CDF as the kernels form it */
    const double t = p < 0.5 ? sqrt(-2.0 * sde_log_tail(p)) : sqrt(-2.0 * sde_log_tail(1.0 - p));
    const double x = t - ((0.010328 * t + 0.802853) * t + 2.515517) /
                             (((0.001308 * t + 0.189269) * t + 1.432788) * t + 1.0);
    return p < 0.5 ? -x : x;
}
"""


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("logtail")
    src = d / "shim.c"
    src.write_text(SHIM)
    so = d / "shim.so"
    subprocess.run([cc, "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-I", HEADER_DIR, str(src), "-o", str(so),
                    "-lm"], check=True)
    L = C.CDLL(str(so))
    L.log_tail_batch.argtypes = [C.c_void_p, C.c_void_p, C.c_long]
    L.as26.argtypes = [C.c_double]
    L.as26.restype = C.c_double
    return L


def _eval(lib, x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty_like(x)
    lib.log_tail_batch(x.ctypes.data, y.ctypes.data, len(x))
    return y


def _points(n, seed):
    rng = np.random.default_rng(seed)
    logu = np.exp2(-rng.uniform(1.0, 1022.0, n // 2))             # log-uniform over the range
    unif = rng.uniform(0.0, 0.5, n - n // 2)                      # the bulk of tail probabilities
    unif = np.maximum(unif, 2.0 ** -60)
    grid = (np.arange(1, 2 ** 12) * 2.0 ** -13)                   # every table slot, below 1/2
    edges = np.array([0.5, np.nextafter(0.5, 0), 0.25, 2.0 ** -53, 2.0 ** -1022, 2.0 ** -33,
                      np.nextafter(0.25, 1), 1.0 / 3, 0.1, 1e-300])
    return np.concatenate([logu, unif, grid, edges])


def test_error_below_0_52_ulp(lib):
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.dps = 60
    x = _points(12000, 1)
    y = _eval(lib, x)
    worst = 0.0
    for xi, yi in zip(x, y):
        t = mpmath.log(mpmath.mpf(float(xi)))
        tf = float(t)
        ulp = math.ulp(tf)
        err = abs(mpmath.mpf(float(yi)) - t) / ulp
        worst = max(worst, float(err))
    assert worst < 0.52, worst


def test_agrees_with_the_c_library(lib):
    x = _points(1_000_000, 2)
    y = _eval(lib, x)
    ref = np.log(x)
    ulps = np.abs(y - ref) / np.spacing(np.abs(ref))
    assert ulps.max() <= 1.0
    # both nearly always return the correctly rounded value
    assert np.mean(y == ref) > 0.999


def test_inverse_cdf_from_it(lib):
    """The AS 26.2.23 normals on this logarithm agree with the C library's
    to 1e-14 (absolute near p = 1/2, where the formula cancels)."""
    rng = np.random.default_rng(3)
    p = np.concatenate([rng.random(20000), [2.0 ** -53, 1 - 2.0 ** -53, 0.5, 1e-10]])
    ours = np.array([lib.as26(float(v)) for v in p])

    def ref(v):
        t = math.sqrt(-2.0 * math.log(v)) if v < 0.5 else math.sqrt(-2.0 * math.log(1.0 - v))
        z = t - ((0.010328 * t + 0.802853) * t + 2.515517) / (((0.001308 * t + 0.189269) * t + 1.432788) * t + 1.0)
        return -z if v < 0.5 else z

    want = np.array([ref(float(v)) for v in p])
    assert np.max(np.abs(ours - want) / np.maximum(np.abs(want), 1.0)) < 1e-14
    assert np.mean(ours == want) > 0.99


def test_outside_the_tail_range_uses_the_library_log(lib):
    x = np.array([0.75, 1.0, 2.0, 1e300, 2.0 ** -1074, 0.0, np.inf])
    with np.errstate(divide="ignore"):
        assert np.array_equal(_eval(lib, x), np.log(x))
    assert np.isnan(_eval(lib, np.array([-1.0, np.nan]))).all()


def test_tables_are_the_generators():
    """The tables in sde_log.h are what gen_log_table.py computes (mpmath)."""
    pytest.importorskip("mpmath")
    import io
    import contextlib
    import importlib.util
    spec = importlib.util.spec_from_file_location("gen_log_table", os.path.join(HEADER_DIR, "gen_log_table.py"))
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        gen.main()
    with open(os.path.join(HEADER_DIR, "sde_log.h")) as f:
        header = f.read()
    assert buf.getvalue().strip() in header
