"""In-tree build of the native libraries (no CMake, no setuptools).

``build()`` compiles
  * ``spike_gb300/libspike_gb300.so``: the sm_103a step engine and its C ABI
    (``csrc/spk_net.cu``), the model-building front end (``csrc/frontend.cpp``)
    and the simulation server (``csrc/spk_server.cpp``);
  * ``oracle/liboracle.so``: the CPU oracle used by the tests and the benchmark's
    CPU baseline (test infrastructure, never linked into the engine).

Float rounding matters for bit-exact parity, so device code is compiled with
``-fmad=false`` (no multiply-add contraction) and host code with
``-ffp-contract=off``.  Translation units are compiled in parallel and only
rebuilt when a source or header is newer than the library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "spike_gb300")
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
ORACLE = os.path.join(ROOT, "oracle")
BUILD_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libspike_gb300.so")
ORACLE_LIB = os.path.join(ORACLE, "liboracle.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-fmad=false", "-std=c++17", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + INCLUDE]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-I" + INCLUDE]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build spike_gb300")


def _cuda_include() -> str:
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(_nvcc()))), "include")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    out = []
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if f.endswith((".h", ".hpp", ".cuh")):
                out.append(os.path.join(d, f))
    return out


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)


def build_engine(force: bool = False) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    units = [
        (os.path.join(CSRC, "spk_net.cu"), os.path.join(BUILD_DIR, "spk_net.o"),
         [nvcc, *ARCH, *NVCC_FLAGS, "-c"]),
        (os.path.join(CSRC, "frontend.cpp"), os.path.join(BUILD_DIR, "frontend.o"),
         ["g++", *CXX_FLAGS, "-c"]),
        (os.path.join(CSRC, "spk_server.cpp"), os.path.join(BUILD_DIR, "spk_server.o"),
         ["g++", *CXX_FLAGS, "-pthread", "-I" + _cuda_include(), "-c"]),
    ]
    todo = [(s, o, c) for (s, o, c) in units if force or _newer(o, [s, *hdrs])]
    with ThreadPoolExecutor(max_workers=len(units)) as ex:
        list(ex.map(lambda u: _run([*u[2], u[0], "-o", u[1]]), todo))
    objs = [o for (_, o, _) in units]
    if force or todo or _newer(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart", "-Xlinker", "-lpthread"])
    return LIB


def build_oracle(force: bool = False) -> str:
    src = os.path.join(ORACLE, "spk_oracle.cpp")
    deps = [src, os.path.join(ORACLE, "spk_oracle.h"), os.path.join(CSRC, "spk_rng.h"),
            os.path.join(INCLUDE, "spike_gb300.h")]
    if force or _newer(ORACLE_LIB, deps):
        _run(["g++", "-std=c++20", "-O3", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
              "-o", ORACLE_LIB, src])
    return ORACLE_LIB


def build_reference_frontend() -> str | None:
    """Compile the reference front end into oracle/_ref with the recipe
    oracle/build_ref.sh (test fixtures only).  The recipe locates the
    reference sources and builds nothing where they are absent."""
    script = os.path.join(ORACLE, "build_ref.sh")
    target = os.path.join(ORACLE, "_ref", "ref_dump")
    deps = [os.path.join(ORACLE, "ref_dump.cpp"), os.path.join(ORACLE, "ref_cases.inc"), script]
    if os.path.exists(target) and not _newer(target, deps):
        return target
    _run(["bash", script])
    return target if os.path.exists(target) else None


def build(force: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_engine, force)
        f2 = ex.submit(build_oracle, force)
        f1.result()
        f2.result()
    build_reference_frontend()


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print("built", LIB, ORACLE_LIB)
