"""The per-pivot tests of the counting kernels against the per-edge tests they stand for.

A one-shot run's kernels decide most edges without double arithmetic: the degree prune is
an integer threshold per pivot degree, and the early stop and the predicate skip use a
float lower bound on the least count either predicate accepts (predicate.cuh: pivot_tests,
edge_pruned, count_floor).  tests/predicate_check.cpp checks, on the host, over 13 million
(eps, dv, du) cases, that the prune equals the reference's 'never' test and its exact
counterpart, and that no count below the bound passes either predicate.  The kernels
compile the same source.
"""
import subprocess

from efficientstructuralgraphclusteringongpus_gb300 import build as pkg_build

HERE = pkg_build.ROOT / "tests"


def test_pivot_tests_match_the_per_edge_tests(tmp_path):
    exe = tmp_path / "predicate_check"
    subprocess.run(["g++", "-O2", "-std=c++17", f"-I{pkg_build.CSRC}", str(HERE / "predicate_check.cpp"), "-o",
                    str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    fields = out.stdout.split()
    assert fields[0] == "ok", out.stdout
    checks, gap0, gap1, gap2, gap3 = map(int, fields[1:])
    assert checks > 10_000_000
    assert gap3 == 0                       # the bound is never more than two below the least count
