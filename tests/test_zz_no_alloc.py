"""The allocation-free butterfly count (bt_bfc_noalloc) through the C ABI.

Some callers may not allocate device memory (plugin hosts that own the device
heap, latency-sensitive paths that cannot afford cudaMalloc); they pass their
own device buffers and the library uses its fixed internal scratch.  The count
must equal the regular entry point's (bt_bfc) exactly, on two calls in a row
(the second call reuses the scratch the first one left behind).

This file is collected last so that, if it fails, a run stopping at the first
failure has already run every other test.
"""

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _device_csr(torch, g):
    off = torch.from_numpy(np.ascontiguousarray(g.offsets).view(np.int32)).cuda()
    nbr = torch.from_numpy(np.ascontiguousarray(g.neighbors).view(np.int32)).cuda()
    return off, nbr


@pytest.mark.parametrize("name", ["aw", "er_config1", "cl20k", "sparse"])
def test_noalloc_count_matches_bt_bfc(engine, name):
    torch = pytest.importorskip("torch")
    gd = load_golden(name)
    g = engine.Graph.from_edges(gd["u"], gd["v"])
    ctx = engine.Context(0)
    try:
        ctx.upload(g)
        expect = ctx.bfc()
    finally:
        ctx.close()
    assert expect == int(gd["bfc"])
    off, nbr = _device_csr(torch, g)
    out = torch.full((1,), -1, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(2):
        engine.bfc_noalloc(0, off.data_ptr(), nbr.data_ptr() if g.m else 0, g.n, g.m,
                           out.data_ptr(), stream.cuda_stream)
        stream.synchronize()
        got = int(out.cpu().numpy().view(np.uint64)[0])
        assert got == expect


def test_noalloc_rejects_oversized_graph(engine):
    torch = pytest.importorskip("torch")
    out = torch.zeros(1, dtype=torch.int64, device="cuda")
    off = torch.zeros(2, dtype=torch.int32, device="cuda")
    with pytest.raises(engine.BitrussError) as ei:
        engine.bfc_noalloc(0, off.data_ptr(), off.data_ptr(), (1 << 22) + 1, 1, out.data_ptr(), 0)
    assert ei.value.code == "BT_ERR_INVALID"
    assert "scratch limit" in str(ei.value)
