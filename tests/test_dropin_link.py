"""The link-level drop-in on the CPU: the reference's own program and types against the engine.

Where the reference sources are present (oracle/build.py builds from them; x86_64, since
its Graph.cpp includes <x86intrin.h>), GPUSCAN++/main.cpp and Graph.cpp, compiled unmodified,
link against libscan_gb300.so in place of GPUScan.cu: the C++ GPUScan symbol it calls
resolves to the engine.  (Running it needs a GPU; the GPU suite runs an equivalent caller.)
The graph_t layout of include/gpuscan_compat.h is compared with the reference's Graph.h.
"""
import subprocess

import pytest

from efficientstructuralgraphclusteringongpus_gb300 import build as pkg_build
from oracle import build as ob

MANGLED = "_Z7GPUScanP7graph_tPiS1_di"


def test_reference_program_links_against_the_engine():
    if not ob.REF_DROPIN.exists():
        pytest.skip("reference sources absent or not x86_64: the reference program was not built")
    undef = subprocess.run(["nm", "-D", "--undefined-only", str(ob.REF_DROPIN)], capture_output=True, text=True,
                           check=True).stdout
    assert MANGLED in undef                       # main.cpp's call, left for the dynamic linker
    libs = subprocess.run(["ldd", str(ob.REF_DROPIN)], capture_output=True, text=True, check=True).stdout
    assert "libscan_gb300.so" in libs and "not found" not in libs
    defined = subprocess.run(["nm", "-D", "--defined-only", str(pkg_build.LIB)], capture_output=True, text=True,
                             check=True).stdout
    assert MANGLED in defined                     # ... which the engine defines


LAYOUT_PROBE = r'''
#include <cstddef>
#include <cstdio>
#include HEADER
int main() {
    std::printf("%zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(graph_t), offsetof(graph_t, n), offsetof(graph_t, m),
                offsetof(graph_t, adj), offsetof(graph_t, num_edges), offsetof(graph_t, eid), sizeof(vid_t),
                sizeof(eid_t));
    return 0;
}
'''


def test_graph_t_layout_matches_reference(tmp_path):
    ref_header = ob.REFERENCE / "Graph.h"
    if not ref_header.exists():
        pytest.skip("reference sources absent")
    src = tmp_path / "probe.cpp"
    src.write_text(LAYOUT_PROBE)
    out = {}
    for name, header, inc in (("reference", '"Graph.h"', ob.REFERENCE), ("engine", '"gpuscan_compat.h"', ob.INCLUDE)):
        exe = tmp_path / name
        # the reference's header uses std::string and uint32_t without including them
        subprocess.run(["g++", "-std=c++14", "-include", "string", "-include", "cstdint", f"-DHEADER={header}",
                        f"-I{inc}", str(src), "-o", str(exe)], check=True)
        out[name] = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert out["reference"] == out["engine"], out
