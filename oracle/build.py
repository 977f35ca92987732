"""Build recipe for the oracle (test infrastructure, never part of the product).

  oracle/_build/liboracle.so       CPU SCAN restatement (scan_oracle.c), gcc + OpenMP
  oracle/_build/libref_harness.so  driver for the reference's own kernels (needs nvcc + a GPU to run)
  oracle/_ref/gpuscan_ref.cubin    the reference's kernels, GPUSCAN++/GPUScan.cu compiled unmodified
  oracle/_ref/libref_graph.so      the reference's host orientation, GPUSCAN++/Graph.cpp compiled
                                   unmodified plus a C shim (only on the machine holding the sources)
  oracle/_ref/ref_convert          the reference's converter, csr_convert/EdgeListToBinsConverter.cpp
  oracle/_ref/gpuscan_dropin       the reference's own program, GPUSCAN++/main.cpp + Graph.cpp compiled
                                   unmodified, linked against libscan_gb300.so instead of GPUScan.cu
                                   (x86_64 only, like libref_graph.so; it needs a GPU to run)

The two oracle/_ref outputs are built from the reference sources where they lie and only
when those sources are present; everything they produce stays out of version control.
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
# Where the reference project's sources lie (read only); SCAN_REFERENCE_ROOT overrides it.
REFERENCE_ROOT = Path(os.environ.get("SCAN_REFERENCE_ROOT", "/root/reference"))
REFERENCE = REFERENCE_ROOT / "GPUSCAN++"
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")

ORACLE_LIB = BUILD / "liboracle.so"
HARNESS_LIB = BUILD / "libref_harness.so"
REF_CUBIN = REF_OUT / "gpuscan_ref.cubin"
REF_GRAPH_LIB = REF_OUT / "libref_graph.so"
REF_CONVERT = REF_OUT / "ref_convert"
REF_DROPIN = REF_OUT / "gpuscan_dropin"
PKG_BUILD = HERE.parent / "efficientstructuralgraphclusteringongpus_gb300" / "_build"
INCLUDE = HERE.parent / "include"
REFERENCE_CONVERT = REFERENCE_ROOT / "csr_convert"


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def _stale(out: Path, *srcs: Path) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(s.exists() and s.stat().st_mtime > t for s in srcs)


def build_oracle() -> Path:
    BUILD.mkdir(exist_ok=True)
    src = HERE / "scan_oracle.c"
    if _stale(ORACLE_LIB, src, Path(__file__)):
        _run(["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", str(src), "-o", str(ORACLE_LIB), "-lm"])
    return ORACLE_LIB


def build_harness() -> Path:
    BUILD.mkdir(exist_ok=True)
    src = HERE / "ref_harness.cu"
    if _stale(HARNESS_LIB, src, Path(__file__)):
        cuda_lib = CUDA_HOME / "lib64"
        _run([NVCC, "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC", str(src), "-o", str(HARNESS_LIB),
              f"-L{cuda_lib}", "-lcuda", "-lcudart"])
    return HARNESS_LIB


def build_reference() -> bool:
    """Compile the reference from its sources (only where they exist).  Returns True if built."""
    if not (REFERENCE / "GPUScan.cu").exists():
        return False
    REF_OUT.mkdir(exist_ok=True)
    # The reference kernels, unmodified, for sm_103a.  -O3 and no -G (its makefile has -g -G).
    # The -include flags supply headers its sources use without including.
    if _stale(REF_CUBIN, REFERENCE / "GPUScan.cu", Path(__file__)):
        _run([NVCC, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17",
              "-include", "string", "-include", "cstdint", "-include", "cstring", f"-I{REFERENCE}",
              str(REFERENCE / "GPUScan.cu"), "-o", str(REF_CUBIN)])
    # The reference's host orientation (getEidAndEdgeList) with a C shim.  Graph.cpp uses
    # <x86intrin.h>, so this only builds on x86_64.
    if platform.machine() == "x86_64" and _stale(REF_GRAPH_LIB, REFERENCE / "Graph.cpp", HERE / "ref_graph_shim.cpp",
                                                Path(__file__)):
        _run(["g++", "-O2", "-std=c++14", "-fPIC", "-shared", "-fopenmp", "-include", "cstdint", "-include",
              "cstring", "-include", "string", f"-I{REFERENCE}", str(REFERENCE / "Graph.cpp"),
              str(HERE / "ref_graph_shim.cpp"), "-o", str(REF_GRAPH_LIB)])
    # The reference's GPUScan program (GPUSCAN++/main.cpp + Graph.cpp, unmodified) with the
    # engine in place of GPUScan.cu: the link-level drop-in of the makefile in INTEGRATION.md.
    lib = PKG_BUILD / "libscan_gb300.so"
    if platform.machine() == "x86_64" and lib.exists() and _stale(
            REF_DROPIN, REFERENCE / "main.cpp", REFERENCE / "Graph.cpp", lib, Path(__file__)):
        _run(["g++", "-O2", "-std=c++14", "-fopenmp", "-include", "cstdint", "-include", "cstring", "-include",
              "string", f"-I{REFERENCE}", str(REFERENCE / "main.cpp"), str(REFERENCE / "Graph.cpp"), "-o",
              str(REF_DROPIN), f"-L{PKG_BUILD}", "-lscan_gb300", f"-Wl,-rpath,{PKG_BUILD}"])
    # The reference's edge-list converter, unmodified (plain C++).
    if (REFERENCE_CONVERT / "EdgeListToBinsConverter.cpp").exists() and _stale(
            REF_CONVERT, REFERENCE_CONVERT / "EdgeListToBinsConverter.cpp", Path(__file__)):
        _run(["g++", "-O2", "-std=c++14", "-include", "algorithm", "-include", "cstdint", f"-I{REFERENCE_CONVERT}",
              str(REFERENCE_CONVERT / "EdgeListToBinsConverter.cpp"), "-o", str(REF_CONVERT)])
    return True


def build_all(with_harness: bool = True) -> None:
    build_oracle()
    build_reference()
    if with_harness:
        build_harness()


if __name__ == "__main__":
    build_all(with_harness="--no-harness" not in sys.argv)
    print("oracle built", file=sys.stderr)
