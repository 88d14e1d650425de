"""Build step of libsdegpu.so (sm_103a).

1. _gen/embedded.h    -- the device runtime headers as C++ raw strings, so
                         NVRTC can compile lowered kernels without a path.
2. _gen/joe_kuo_d6.h  -- the Joe-Kuo D6 table (21201 dimensions; the data
                         the sobol crate embeds), read from scipy's copy.
3. nvcc / g++ in parallel, linked into sde_sim_rs/libsdegpu.so.

Run on the machine that will load the library (x86_64 here, aarch64 on the
GPU hosts); nvcc cross-compiles sm_103a device code without a GPU.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.normpath(os.path.join(HERE, "..", "sde_sim_rs"))
GEN = os.path.join(HERE, "_gen")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(PKG, "libsdegpu.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def cuda_home() -> str:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _write_if_changed(path: str, text: str) -> None:
    if os.path.exists(path):
        with open(path) as f:
            if f.read() == text:
                return
    with open(path, "w") as f:
        f.write(text)


def gen_embedded() -> None:
    out = ["// generated by build.py -- do not edit", "#pragma once"]
    for name, rel in (("kEmbArgs", "device/sde_args.h"), ("kEmbLog", "device/sde_log.h"), ("kEmbChacha", "device/sde_chacha.h"), ("kEmbShift", "device/sde_shift.h"),
                      ("kEmbRt", "device/sde_rt.cuh")):
        with open(os.path.join(HERE, rel)) as f:
            text = f.read()
        assert ")SDEEMB\"" not in text
        out.append(f'static const char {name}[] = R"SDEEMB(\n{text})SDEEMB";')
    _write_if_changed(os.path.join(GEN, "embedded.h"), "\n".join(out) + "\n")


def gen_joe_kuo() -> None:
    path = os.path.join(GEN, "joe_kuo_d6.h")
    if os.path.exists(path):
        return
    import numpy as np
    import scipy.stats as st
    npz = os.path.join(os.path.dirname(st.__file__), "_sobol_direction_numbers.npz")
    d = np.load(npz)
    poly = d["poly"].astype(np.int64)
    vinit = d["vinit"].astype(np.int64)
    assert poly.shape[0] == vinit.shape[0] and vinit.shape[1] == 18
    assert poly.max() < 2**32 and vinit.max() < 2**32
    lines = ["// generated by build.py from the Joe-Kuo D6 table -- do not edit",
             "#pragma once", "#include <cstdint>",
             f"static const int kJkDims = {poly.shape[0]};",
             "static const uint32_t kJkPoly[] = {"]
    for i in range(0, len(poly), 16):
        lines.append(",".join(str(int(x)) for x in poly[i:i + 16]) + ",")
    lines.append("};")
    lines.append("static const uint32_t kJkVinit[] = {")
    flat = vinit.reshape(-1)
    for i in range(0, len(flat), 36):
        lines.append(",".join(str(int(x)) for x in flat[i:i + 36]) + ",")
    lines.append("};")
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        f.write("\n".join(lines) + "\n")
    os.replace(tmp, path)


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False) -> str:
    os.makedirs(GEN, exist_ok=True)
    os.makedirs(OBJ, exist_ok=True)
    gen_embedded()
    gen_joe_kuo()
    cuda = cuda_home()
    inc = ["-I" + os.path.join(cuda, "include"), "-I" + HERE]
    headers = [os.path.join(HERE, h) for h in
               ("frontend.h", "codegen.h", "kernels.h", "device/sde_args.h", "device/sde_log.h", "device/sde_chacha.h", "device/sde_shift.h", "device/sde_rt.cuh",
                "_gen/embedded.h", "_gen/joe_kuo_d6.h")]
    headers.append(os.path.normpath(os.path.join(HERE, "..", "..", "include", "sdegpu.h")))
    jobs = []
    objs = []
    for src in ("frontend.cpp", "codegen.cpp", "engine.cpp"):
        o = os.path.join(OBJ, src.replace(".cpp", ".o"))
        objs.append(o)
        s = os.path.join(HERE, src)
        if _stale(o, [s] + headers + [os.path.abspath(__file__)]):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function",
                         *inc, "-c", s, "-o", o])
    for src in ("kernels.cu", "noalloc.cu"):
        o = os.path.join(OBJ, src.replace(".cu", ".o"))
        objs.append(o)
        s = os.path.join(HERE, src)
        if _stale(o, [s] + headers + [os.path.join(HERE, "engine_internal.h"), os.path.abspath(__file__)]):
            # -fmad=false: the known-answer kernels evaluate the FP64 inverse
            # CDF exactly as the lowered FP64 kernels do (no contraction)
            jobs.append(["nvcc", ARCH, "-O3", "-fmad=false", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         *inc, "-c", s, "-o", o])
    procs = [(j, subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
             for j in jobs]
    failed = []
    for j, p in procs:
        out, _ = p.communicate()
        if verbose and out:
            print(out)
        if p.returncode != 0:
            failed.append((j, out))
    if failed:
        msg = "\n".join(" ".join(j) + "\n" + out for j, out in failed)
        raise RuntimeError("libsdegpu build failed:\n" + msg)
    if jobs or not os.path.exists(LIB):
        libdir = os.path.join(cuda, "lib64")
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = ["nvcc", ARCH, "-shared", "-cudart", "shared", "-o", tmp, *objs,
               "-L" + libdir, "-lnvrtc", "-Xlinker", "-rpath," + libdir]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError("libsdegpu link failed:\n" + " ".join(cmd) + "\n" + r.stdout)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
