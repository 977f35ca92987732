"""Build recipe for libscan_gb300.so and the `gpuscan` CLI (in-tree, under _build/).

Host C++ is compiled with g++ (C++17, OpenMP), device code with nvcc for sm_103a only.
Translation units compile in parallel; a stamp of sources + flags skips unchanged builds.
No CMake: the tool chain is nvcc + g++, the same on x86_64 and aarch64 hosts.
"""
from __future__ import annotations

import hashlib
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = BUILD / "libscan_gb300.so"
CLI = BUILD / "gpuscan"
CONVERT_CLI = BUILD / "scan-convert"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CXXFLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-Wall", "-Wno-unused-function", f"-I{INCLUDE}", f"-I{CSRC}"]
NVCCFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-fopenmp", f"-I{INCLUDE}", f"-I{CSRC}",
                    "-Xptxas", "-warn-spills"]

CXX_SOURCES = ["graph.cpp", "compat.cpp"]
CU_SOURCES = ["scan_device.cu", "noalloc.cu", "server.cu", "batch.cu"]
HEADERS = ["graph_internal.h", "device_common.cuh", "device_graph.h", "predicate.cuh", "kernels_orient.cuh", "kernels_cn.cuh", "kernels_cluster.cuh"]


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def _stamp() -> str:
    h = hashlib.sha256()
    for name in CXX_SOURCES + CU_SOURCES + HEADERS + ["cli.cpp", "convert_cli.cpp"]:
        h.update((CSRC / name).read_bytes())
    for hdr in sorted(INCLUDE.glob("*.h")):
        h.update(hdr.read_bytes())
    h.update(" ".join(CXXFLAGS + NVCCFLAGS).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile the library and CLI if sources changed; return the library path."""
    BUILD.mkdir(exist_ok=True)
    stamp_file = BUILD / "stamp"
    stamp = _stamp()
    if (not force and LIB.exists() and CLI.exists() and CONVERT_CLI.exists() and stamp_file.exists()
            and stamp_file.read_text() == stamp):
        return LIB
    jobs = []
    objs = []
    for src in CXX_SOURCES:
        obj = BUILD / (Path(src).stem + ".o")
        jobs.append(["g++", *CXXFLAGS, "-c", str(CSRC / src), "-o", str(obj)])
        objs.append(obj)
    for src in CU_SOURCES:
        obj = BUILD / (Path(src).stem + ".cu.o")
        jobs.append([NVCC, *NVCCFLAGS, "-c", str(CSRC / src), "-o", str(obj)])
        objs.append(obj)
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(_run, jobs))
    cuda_lib = CUDA_HOME / "lib64"
    if not (cuda_lib / "libcudart.so").exists():
        cuda_lib = CUDA_HOME / "targets" / f"{os.uname().machine}-linux" / "lib"
    _run(["g++", "-shared", "-o", str(LIB), *map(str, objs), f"-L{cuda_lib}", "-lcudart", "-fopenmp",
          f"-Wl,-rpath,{cuda_lib}", "-Wl,--no-undefined"])
    for src, exe in (("cli.cpp", CLI), ("convert_cli.cpp", CONVERT_CLI)):
        _run(["g++", "-O2", "-std=c++17", f"-I{INCLUDE}", str(CSRC / src), "-o", str(exe), f"-L{BUILD}",
              "-lscan_gb300", "-Wl,-rpath,$ORIGIN"])
    stamp_file.write_text(stamp)
    if verbose:
        print(f"built {LIB} and {CLI}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
