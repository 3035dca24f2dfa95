"""Build recipes for the native parts of alens_gb300.

* ``build_lib()`` compiles the CUDA library ``alens_gb300/lib/libalens_gpu.so``
  (kernels + C ABI of ``include/alens_gpu.h``) for sm_103a with nvcc.
* ``build_oracle()`` compiles the CPU oracle ``oracle/liboracle.so`` with g++
  (test infrastructure; the library never links it).
* ``build_facade_driver()`` compiles the C++ ``SylinderSystem`` facade demo
  driver against the library.

Everything is built in-tree, one translation unit per process, in parallel.
Host code uses no architecture-specific flags so that the same sources build
on x86-64 and aarch64 hosts.
"""
from __future__ import annotations

import concurrent.futures as _fut
import os
import shutil
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "alens_gb300"
CSRC = PKG / "csrc"
LIBDIR = PKG / "lib"
BUILDDIR = PKG / "_build"
ORACLE = ROOT / "oracle"

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
if not Path(NVCC).exists():
    NVCC = shutil.which("nvcc") or NVCC
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]

# Translation units of the GPU library.  Files listed in FP_STRICT hold the
# FP64 path that must match the oracle bit for bit: they are compiled without
# FMA contraction.
CU_SOURCES = ["engine.cu", "kernels_detect.cu", "kernels_assemble.cu", "kernels_solve.cu",
              "kernels_mixed.cu", "kernels_fast.cu", "kernels_csm.cu", "kernels_mlp.cu", "mlp.cu", "kernels_noalloc.cu", "kernels_kmc.cu", "capi.cu"]
CXX_SOURCES: list[str] = []
FP_STRICT = {"kernels_detect.cu", "kernels_assemble.cu", "kernels_solve.cu", "kernels_noalloc.cu",
             "kernels_kmc.cu", "engine.cu", "capi.cu"}


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                          text=True)
    if proc.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + proc.stdout)


def _newer(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(d.stat().st_mtime <= t for d in deps if d.exists())


def lib_path() -> Path:
    return LIBDIR / "libalens_gpu.so"


def oracle_path() -> Path:
    return ORACLE / "liboracle.so"


def build_oracle(force: bool = False) -> Path:
    out = oracle_path()
    deps = [ORACLE / "oracle.cpp", ORACLE / "oracle_kmc.cpp", ORACLE / "oracle.h", ORACLE / "oracle_ctx.h",
            ROOT / "include" / "alens_gpu.h"]
    if not force and _newer(out, deps):
        return out
    cxx = os.environ.get("CXX", "g++")
    _run([cxx, "-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC",
          "-shared", "-Wall", "-Wextra", "-Wno-unused-parameter",
          "-I", str(ROOT / "include"), str(ORACLE / "oracle.cpp"), str(ORACLE / "oracle_kmc.cpp"), "-o", str(out)])
    return out


def _compile_cu(src: str) -> Path:
    obj = BUILDDIR / (src + ".o")
    flags = [NVCC, *GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
             "-Xcompiler", "-ffp-contract=off",
             "-I", str(ROOT / "include"), "-I", str(CSRC), "-c", str(CSRC / src), "-o", str(obj)]
    if src in FP_STRICT:
        flags.insert(3, "--fmad=false")
    if os.environ.get("ALENS_PTXAS_VERBOSE"):
        flags += ["-Xptxas", "-v"]
    extra = os.environ.get("ALENS_NVCC_FLAGS", "").split()
    if extra:
        flags += extra
    _run(flags)
    return obj


def build_lib(force: bool = False, jobs: int | None = None) -> Path:
    out = lib_path()
    srcs = [CSRC / s for s in CU_SOURCES + CXX_SOURCES]
    hdrs = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + [ROOT / "include" / "alens_gpu.h"]
    if not force and _newer(out, srcs + hdrs):
        return out
    BUILDDIR.mkdir(parents=True, exist_ok=True)
    LIBDIR.mkdir(parents=True, exist_ok=True)
    jobs = jobs or min(len(CU_SOURCES), os.cpu_count() or 4)
    with _fut.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(_compile_cu, CU_SOURCES))
    _run([NVCC, *GENCODE, "-shared", "-o", str(out), *map(str, objs), "-lcudart"])
    return out


def build_facade_driver(force: bool = False) -> Path:
    """C++ demo driver that steps a system through the SylinderSystem facade."""
    out = LIBDIR / "facade_driver"
    src = CSRC / "facade" / "facade_driver.cpp"
    deps = [src, CSRC / "facade" / "SylinderSystem.hpp", CSRC / "facade" / "SylinderSystem.cpp",
            lib_path()]
    if not force and _newer(out, deps):
        return out
    cxx = os.environ.get("CXX", "g++")
    # no FMA contraction: aarch64 g++ contracts a*b+c by default, which would
    # round the reader's lengths and quaternions differently from the oracle
    _run([cxx, "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-Wall", "-I", str(ROOT / "include"),
          "-I", str(CSRC / "facade"),
          str(src), str(CSRC / "facade" / "SylinderSystem.cpp"),
          "-L", str(LIBDIR), "-lalens_gpu", "-Wl,-rpath," + str(LIBDIR), "-o", str(out)])
    return out


def build_all(force: bool = False) -> None:
    with _fut.ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_oracle, force)
        f2 = ex.submit(build_lib, force)
        f1.result()
        f2.result()
    if (CSRC / "facade" / "facade_driver.cpp").exists():
        build_facade_driver(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print("built", lib_path(), oracle_path())
