"""The allocation-free core check, scan_cores_noalloc, against scan_run's cores.

scan_cores_noalloc serves callers that may not allocate device memory themselves (a
plugin or custom call whose framework owns all device memory, a process whose HBM is
committed to resident graphs, code that must avoid cudaMalloc's device-wide
synchronisation).  Its scratch is a fixed array inside the library, shared by every call.
This test gives it device buffers (allocated here with torch, standing in for the
caller's memory) and checks two calls in a row against scan_run; the first call is the
permissive one, so counts left behind in the shared scratch would show up in the second.
"""
import numpy as np
import pytest

import efficientstructuralgraphclusteringongpus_gb300 as sg

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def device_buffers(g):
    _, eu, ev = g.orient_reference()
    cn, _ = g.common_neighbors()
    dev = torch.device("cuda", 0)
    as_dev = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).to(dev)
    return {
        "off": as_dev(g.offsets().astype(np.uint32)),
        "eu": as_dev(eu.astype(np.uint32)),
        "ev": as_dev(ev.astype(np.uint32)),
        "cn": as_dev(cn.astype(np.uint32)),
        "E": int(cn.size),
    }


def noalloc_cores(g, bufs, eps, mu, mode):
    out = torch.full((g.n,), 7, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    sg.cores_noalloc(bufs["off"].data_ptr(), g.n, bufs["eu"].data_ptr(), bufs["ev"].data_ptr(),
                     bufs["cn"].data_ptr(), bufs["E"], eps, mu, mode, out.data_ptr(), stream)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("make", [
    lambda: sg.Graph.sbm(5000, 8, 0.1, 0.001, 64, seed=3),
    lambda: sg.Graph.rmat(14, 16, seed=5),
], ids=["sbm5000", "rmat14"])
def test_noalloc_cores_match_scan_run_on_two_calls(make):
    g = make()
    bufs = device_buffers(g)
    # permissive first, strict second
    for eps, mu, mode in (("0.1", 2, sg.PRED_EXACT), ("0.6", 4, sg.PRED_REF_F64)):
        expect = (g.run(eps, mu, mode).role == sg.ROLE_CORE).astype(np.uint8)
        got = noalloc_cores(g, bufs, eps, mu, mode)
        assert np.array_equal(got, expect), (eps, mu, int((got != expect).sum()))
    assert expect.sum() < (g.run("0.1", 2, sg.PRED_EXACT).role == sg.ROLE_CORE).sum()


def test_noalloc_rejects_graphs_above_its_scratch():
    with pytest.raises(sg.ScanError) as e:
        sg.cores_noalloc(16, (1 << 20) + 1, 16, 16, 16, 1, "0.5", 2, sg.PRED_EXACT, 16, 0)
    assert e.value.status == 6 and "at most 1048576 vertices" in str(e.value)
