"""The C++ GPUScan symbol called for real: a C++ program written to the reference's
interface (tests/gpuscan_caller.cpp follows GPUSCAN++/main.cpp:20-123) is compiled against
the library and include/, run on a b_degree.bin/b_adj.bin folder, and its labels and its
"Cluster Number" line are compared with the oracle (ref-f64, the predicate GPUScan() uses).
"""
import subprocess
from pathlib import Path

import numpy as np
import pytest

import efficientstructuralgraphclusteringongpus_gb300 as sg
from efficientstructuralgraphclusteringongpus_gb300 import build as pkg_build
from oracle import oracle

pytestmark = pytest.mark.gpu

HERE = Path(__file__).resolve().parent


@pytest.fixture(scope="module")
def caller(tmp_path_factory):
    exe = tmp_path_factory.mktemp("caller") / "gpuscan_caller"
    subprocess.run(["g++", "-O2", "-std=c++17", f"-I{pkg_build.INCLUDE}", str(HERE / "gpuscan_caller.cpp"), "-o",
                    str(exe), f"-L{pkg_build.BUILD}", "-lscan_gb300", f"-Wl,-rpath,{pkg_build.BUILD}"], check=True)
    return exe


@pytest.mark.parametrize("scale,seed,eps,mu", [(16, 1, "0.5", 5), (14, 2, "0.3", 3), (12, 4, "0.4", 2)])
def test_cpp_gpuscan_symbol_matches_oracle(caller, tmp_path, scale, seed, eps, mu):
    g = sg.Graph.rmat(scale, 16, seed=seed)
    g.save(tmp_path / "g")
    out = tmp_path / "labels.bin"
    p = subprocess.run([str(caller), str(tmp_path / "g"), eps, str(mu), str(out)], capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
    label, _, counts = oracle.scan(g.offsets(), g.adjacency(), eps, mu, 1)
    assert np.array_equal(np.fromfile(out, dtype=np.int32), label)
    assert f"Cluster Number: {counts['clusters']}" in p.stderr
