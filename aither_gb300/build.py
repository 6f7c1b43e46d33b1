"""In-tree build of the native library and the CPU oracle.

``python -m aither_gb300.build`` compiles
  * aither_gb300/libaither_gb300.so  -- host setup (C++) + sm_103a kernels
    (CUDA) behind the C ABI of include/aither_gb300.h;
  * oracle/liboracle.so               -- the CPU oracle (plain C), test
    infrastructure only;
  * oracle/_ref/                      -- when the reference sources are
    present on this machine, the reference solver built as an oracle.

Translation units compile in parallel; one -gencode (sm_103a).  FP64
kernels are compiled with --fmad=false so every multiply and add rounds like
the reference's host build (-ffp-contract=off).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "aither_gb300")
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build", platform.machine())
LIB = os.path.join(PKG, "libaither_gb300.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "liboracle.so")
REF_BUILD = os.path.join(ORACLE_DIR, "ref_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")

# .cu units and their arithmetic flags
CU_UNITS = {
    "kernels_fp64.cu": ["--fmad=false"],
    "kernels_fp64_fast.cu": ["--fmad=true"],
    "kernels_fp32.cu": ["--fmad=true"],
    "batch.cu": ["--fmad=false"],
    "noalloc.cu": ["--fmad=false"],
    "geometry.cu": ["--fmad=false"],
}
CPP_UNITS = ["setup.cpp", "capi_setup.cpp", "output.cpp"]


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    out = cmd[cmd.index("-o") + 1] if "-o" in cmd else None
    if out:
        with open(out + ".arch", "w") as f:
            f.write(platform.machine())


def _stale(target: str, deps: list[str]) -> bool:
    """True when target is missing, older than a dependency, or was built
    for another machine architecture (a copied tree keeps foreign builds)."""
    if not os.path.exists(target):
        return True
    stamp = target + ".arch"
    if not os.path.exists(stamp) or open(stamp).read().strip() != platform.machine():
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _headers() -> list[str]:
    hs = [os.path.join(ROOT, "include", "aither_gb300.h")]
    for f in os.listdir(CSRC):
        if f.endswith((".hpp", ".cuh", ".h")):
            hs.append(os.path.join(CSRC, f))
    return hs


def build_library(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    jobs = []
    objs = []
    hdrs = _headers()
    for cu, flags in CU_UNITS.items():
        src = os.path.join(CSRC, cu)
        if not os.path.exists(src):
            continue
        obj = os.path.join(BUILD, cu + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            jobs.append([NVCC, *ARCH, "-lineinfo", "-O3", "-std=c++17", *flags,
                         "-Xcompiler", "-fPIC", "-Xptxas", "-v", *inc, "-c", src, "-o", obj])
    for cpp in CPP_UNITS:
        src = os.path.join(CSRC, cpp)
        obj = os.path.join(BUILD, cpp + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off",
                         "-Wall", *inc, "-I" + os.path.join(CUDA_HOME, "include"),
                         "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(len(jobs), 1)) as ex:
        list(ex.map(_run, jobs))
    if _stale(LIB, objs):
        _run([NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    return LIB


def build_oracle() -> str:
    src = os.path.join(ORACLE_DIR, "aither_oracle.c")
    deps = [src, os.path.join(ORACLE_DIR, "aither_oracle.h"),
            os.path.join(ROOT, "include", "aither_gb300.h")]
    if _stale(ORACLE_LIB, deps):
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off",
              "-fopenmp", "-I" + os.path.join(ROOT, "include"), src, "-o", ORACLE_LIB, "-lm"])
    return ORACLE_LIB


def reference_source() -> str | None:
    """The reference's source tree: AITHER_REFERENCE_SRC, else the default
    of the oracle/ref_build recipe; None where neither holds its sources
    (machines that only receive prebuilt files)."""
    ref = os.environ.get("AITHER_REFERENCE_SRC")
    if not ref:
        r = subprocess.run(["make", "-s", "-C", REF_BUILD, "print-ref"], capture_output=True,
                           text=True)
        ref = r.stdout.strip() if r.returncode == 0 else ""
    return ref if ref and os.path.isdir(os.path.join(ref, "src")) else None


def build_reference(ref: str | None = None, jobs: int = 8) -> str | None:
    """Builds the reference solver from its sources in place (only where the
    sources exist)."""
    ref = ref or reference_source()
    if ref is None:
        return None
    out = os.path.join(ORACLE_DIR, "_ref")
    _run(["make", "-C", REF_BUILD, f"REF={ref}", f"OUT={out}", f"-j{jobs}"])
    return out


def build_all(with_reference: bool = True) -> None:
    build_library()
    build_oracle()
    if with_reference:
        build_reference()


if __name__ == "__main__":
    build_all(with_reference="--no-ref" not in sys.argv)
    print("built", LIB, ORACLE_LIB)
