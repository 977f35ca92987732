"""Generates the golden fixtures under tests/golden/ from the reference's own code.

  --orient   (CPU; needs the reference sources, compiled by oracle/build.py into
             oracle/_ref/libref_graph.so) -> orient_<name>.npz:
             CSR + eid / Edge_u / Edge_v from GPUSCAN++/Graph.cpp:52-141 (getEidAndEdgeList).
  --convert  (CPU; needs oracle/_ref/ref_convert, csr_convert/EdgeListToBinsConverter.cpp built from
             the reference sources) -> convert_edges.txt + convert_b_degree.bin / convert_b_adj.bin:
             an edge list (comments, both directions, a self-loop) and the converter's output.
  --kernels  (GPU; needs oracle/_ref/gpuscan_ref.cubin, the reference's GPUScan.cu kernels)
             -> refgpu_<name>.npz: CSR + the reference's result array for several (eps, mu),
             produced by oracle/ref_harness.cu replaying GPUScan() (GPUSCAN++/GPUScan.cu:800-1009).

  python tests/golden/make_golden.py --orient --kernels [--out DIR]

The graphs are small (hand-built, R-MAT scale 8/10, an SBM) so the fixtures stay a few
hundred KB.  Fixtures are self-contained: they store the CSR, so tests do not depend on the
generator staying bit-identical.
"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import efficientstructuralgraphclusteringongpus_gb300 as sg  # noqa: E402
from oracle import oracle  # noqa: E402

PARAMS = [("0.2", 2), ("0.4", 2), ("0.4", 5), ("0.5", 3), ("0.5", 5), ("0.6", 2), ("0.8", 3)]


def graphs() -> dict:
    a = [(i, j) for i in range(7) for j in range(i + 1, 7)]
    b = [(i, j) for i in range(8, 15) for j in range(i + 1, 15)]
    ring = [(i, (i + 1) % 20) for i in range(20)] + [(i, (i + 5) % 20) for i in range(20)]
    return {
        "cliques": sg.Graph.from_edges(18, a + b + [(7, 5), (7, 6), (7, 8), (7, 9), (15, 0), (15, 14), (16, 3),
                                                    (16, 10), (17, 2)]),
        "ring4": sg.Graph.from_edges(20, ring),
        "star": sg.Graph.from_edges(40, [(0, i) for i in range(1, 40)] + [(1, 2), (2, 3)]),
        "rmat8": sg.Graph.rmat(8, 16, seed=1),
        "rmat10": sg.Graph.rmat(10, 16, seed=2),
        "sbm": sg.Graph.sbm(600, 6, 0.2, 0.005, 64, seed=4),
    }


def make_orient(out: Path) -> None:
    if not oracle.reference_orientation_available():
        raise SystemExit("reference orientation library missing (build oracle/_ref first)")
    for name, g in graphs().items():
        off, adj = g.offsets(), g.adjacency()
        eid, eu, ev = oracle.reference_orient(off, adj)
        np.savez_compressed(out / f"orient_{name}.npz", offsets=off, adj=adj, eid=eid, edge_u=eu, edge_v=ev)
        print("wrote", out / f"orient_{name}.npz")


def convert_edge_list_text() -> str:
    g = sg.Graph.rmat(9, 8, seed=4)
    off, adj = g.offsets(), g.adjacency()
    lines = ["# synthetic edge list: both directions of each edge, a self-loop, a comment"]
    for v in range(g.n):
        for w in adj[off[v]:off[v + 1]]:
            lines.append(f"{v} {w}")
    lines.insert(5, "7 7")
    return "\n".join(lines) + "\n"


def make_convert(out: Path) -> None:
    import subprocess
    import tempfile

    from oracle import build as ob
    if not ob.REF_CONVERT.exists():
        raise SystemExit("reference converter missing (build oracle/_ref first)")
    text = convert_edge_list_text()
    (out / "convert_edges.txt").write_text(text)
    with tempfile.TemporaryDirectory() as tmp:
        subprocess.run([str(ob.REF_CONVERT), str(out / "convert_edges.txt"), f"{tmp}/deg", f"{tmp}/adj"], check=True,
                       stdout=subprocess.DEVNULL)
        (out / "convert_b_degree.bin").write_bytes(Path(f"{tmp}/deg").read_bytes())
        (out / "convert_b_adj.bin").write_bytes(Path(f"{tmp}/adj").read_bytes())
    print("wrote", out / "convert_b_degree.bin")


def make_kernels(out: Path) -> None:
    if not oracle.reference_kernels_available():
        raise SystemExit("reference cubin missing (build oracle/_ref first)")
    for name, g in graphs().items():
        off, adj = g.offsets(), g.adjacency()
        results = {}
        for eps, mu in PARAMS:
            ref, _ = oracle.reference_gpuscan(off, adj, float(eps), mu)
            results[f"eps{eps}_mu{mu}"] = ref
        np.savez_compressed(out / f"refgpu_{name}.npz", offsets=off, adj=adj,
                            params=np.array([f"{e}:{m}" for e, m in PARAMS]), **results)
        print("wrote", out / f"refgpu_{name}.npz")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--orient", action="store_true")
    ap.add_argument("--kernels", action="store_true")
    ap.add_argument("--convert", action="store_true")
    ap.add_argument("--out", default=str(Path(__file__).resolve().parent))
    a = ap.parse_args()
    out = Path(a.out)
    out.mkdir(parents=True, exist_ok=True)
    if a.orient:
        make_orient(out)
    if a.convert:
        make_convert(out)
    if a.kernels:
        make_kernels(out)


if __name__ == "__main__":
    main()
