"""Builds the CUDA library in-tree (sm_103a only).

    python -m spoa_gb300.build

Compiles the four translation units in parallel with nvcc and links
spoa_gb300/libspoa_gb300.so (the C ABI of include/spoa_gb300.h), then the C++
drop-in layer spoa_gb300/libspoa.so (include/spoa/*.hpp) and the `spoa`
command-line program spoa_gb300/spoa over it.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libspoa_gb300.so")
CPPLIB = os.path.join(HERE, "libspoa.so")
PEAKLIB = os.path.join(HERE, "libspoa_peak.so")
CPPTEST = os.path.join(OUT, "spoa_api_test")
CLI = os.path.join(HERE, "spoa")

TUS = ["spoa_gb300"] + [f"inst_{m}{w}" for m in ("linear", "affine", "convex") for w in (16, 32)]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise FileNotFoundError("nvcc not found")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return hs + [os.path.join(ROOT, "include", "spoa_gb300.h")]


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    hdrs = _headers()
    flags = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                    "-I", os.path.join(ROOT, "include")]

    def compile_one(tu: str) -> str:
        src = os.path.join(CSRC, tu + ".cu")
        obj = os.path.join(OUT, tu + ".o")
        if force or _stale(obj, [src] + hdrs):
            cmd = [cc] + flags + ["-c", src, "-o", obj]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed for {tu}:\n{r.stderr}")
            if verbose:
                print(r.stderr, file=sys.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(TUS)) as ex:
        objs = list(ex.map(compile_one, TUS))
    if force or _stale(LIB, objs):
        subprocess.run([cc] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs, check=True)
    # integer-pipe peak probe used by the benchmark (not part of the C ABI)
    peak_src = os.path.join(CSRC, "int_peak.cu")
    if force or _stale(PEAKLIB, [peak_src]):
        subprocess.run([cc] + ARCH + ["-O3", "-Xcompiler", "-fPIC", "-shared", "-cudart",
                                      "static", peak_src, "-o", PEAKLIB], check=True)
    # C++ drop-in layer over the C ABI
    cpp_src = os.path.join(CSRC, "spoa_api.cpp")
    if os.path.exists(cpp_src):
        cpp_hdrs = [os.path.join(ROOT, "include", "spoa", f)
                    for f in os.listdir(os.path.join(ROOT, "include", "spoa"))]
        if force or _stale(CPPLIB, [cpp_src, LIB] + cpp_hdrs + hdrs):
            subprocess.run(["g++", "-std=c++11", "-O2", "-Wall", "-fPIC", "-shared",
                            "-I", os.path.join(ROOT, "include"), cpp_src, "-o", CPPLIB,
                            "-L", HERE, "-lspoa_gb300", "-Wl,-rpath,$ORIGIN"], check=True)
        # the C++ API test driver (tests/test_cpp_api.py runs it)
        test_src = os.path.join(ROOT, "tests", "cpp", "spoa_api_test.cpp")
        if os.path.exists(test_src) and (force or _stale(CPPTEST, [test_src, CPPLIB] + cpp_hdrs)):
            subprocess.run(["g++", "-std=c++11", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
                            test_src, "-o", CPPTEST, "-L", HERE, "-lspoa",
                            "-Wl,-rpath," + HERE], check=True)
        # the spoa command-line program (gzip input where zlib is installed)
        cli_src = os.path.join(CSRC, "spoa_cli.cpp")
        if os.path.exists(cli_src) and (force or _stale(CLI, [cli_src, CPPLIB] + cpp_hdrs)):
            zlib = subprocess.run(["g++", "-x", "c++", "-E", "-"], input="#include <zlib.h>\n",
                                  capture_output=True, text=True).returncode == 0
            subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
                            cli_src, "-o", CLI, "-L", HERE, "-lspoa", "-lspoa_gb300"]
                           + (["-lz"] if zlib else []) + ["-Wl,-rpath,$ORIGIN"], check=True)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
