"""Serving loop: admission against an HBM budget, continuous batching, and
the identity of every result alone and in a mix of concurrent requests."""

import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden
from test_batch import random_lists


def golden_graphs(engine):
    gds = [load_golden(n) for n in GOLDEN_CASES]
    return gds, [engine.Graph.from_edges(gd["u"], gd["v"]) for gd in gds]


def test_server_needs_a_device(engine):
    """Without a GB300 the server fails to start with a status, not a crash."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(engine.BitrussError) as ei:
        engine.Server(0, 2, 0)
    assert ei.value.code == "BT_ERR_NO_DEVICE"


@pytest.mark.gpu
def test_results_same_alone_and_in_mix(engine, oracle_mod):
    O = oracle_mod
    gds, graphs = golden_graphs(engine)
    rnd = random_lists(24, 21)
    rgraphs = [engine.Graph.from_edges(u, v) for u, v in rnd]
    allg = graphs + rgraphs
    ops = ["msp", "ebfc", "bfc", "msp_exact"]
    rng = np.random.default_rng(3)
    work = [(i, op) for i in range(len(allg)) for op in ops]
    # alone: one slot, one request in flight at a time
    alone = {}
    srv = engine.Server(0, 1, 0)
    try:
        for i, op in work:
            t, out = srv.submit(allg[i], op)
            info = srv.wait(t)
            assert info["status"] == 0 and info["batch_size"] == 1
            alone[(i, op)] = (None if out is None else out.copy(), info["count"], info["levels"])
    finally:
        srv.close()
    # in a mix: three slots, every request queued at once, shuffled
    order = [work[k] for k in rng.permutation(len(work))]
    srv = engine.Server(0, 3, 0)
    try:
        tickets = [(key, *srv.submit(allg[key[0]], key[1])) for key in order]
        batched = 0
        for key, t, out in tickets:
            info = srv.wait(t)
            assert info["status"] == 0
            batched += info["batch_size"] > 1
            a_out, a_count, a_levels = alone[key]
            if out is not None:
                np.testing.assert_array_equal(out, a_out)
            if key[1] in ("bfc", "ebfc"):
                assert info["count"] == a_count
            else:
                assert info["levels"] == a_levels
        st = srv.stats()
        assert batched > 0 and st["batches"] > 0
        p50, p99, n = srv.latency()
        assert n == len(work) and 0 < p50 <= p99
    finally:
        srv.close()
    # and both equal the reference / oracle
    for i, g in enumerate(allg):
        if i < len(gds):
            gd = gds[i]
            np.testing.assert_array_equal(alone[(i, "msp")][0][:g.m].astype(np.uint64), gd["msp"])
            np.testing.assert_array_equal(alone[(i, "msp_exact")][0][:g.m].astype(np.uint64), gd["hidx"])
            np.testing.assert_array_equal(alone[(i, "ebfc")][0][:g.m], gd["ebfc"])
            assert alone[(i, "bfc")][1] == int(gd["count"])
        else:
            d = O.build_csr(*rnd[i - len(gds)])
            want, lv, _ = O.msp(d, 0, O.MSP_REF)
            np.testing.assert_array_equal(alone[(i, "msp")][0][:g.m].astype(np.uint64), want)
            assert alone[(i, "msp")][2] == lv


@pytest.mark.gpu
def test_admission_budget(engine, gpu_ctx):
    gd = load_golden("cl20k")
    g = engine.Graph.from_edges(gd["u"], gd["v"])
    need = gpu_ctx.job_bytes([g], "msp")
    need2 = gpu_ctx.job_bytes([g, g], "msp")
    assert need2 > need
    # room for one such job at a time (not for a batch of two): every request
    # still completes, in turn
    srv = engine.Server(0, 4, (need + need2) // 2)
    try:
        ts = [srv.submit(g, "msp") for _ in range(6)]
        for t, out in ts:
            info = srv.wait(t)
            np.testing.assert_array_equal(out.astype(np.uint64), gd["msp"])
            assert info["batch_size"] == 1  # two would not fit
    finally:
        srv.close()
    # a request larger than the whole budget fails with a status
    srv = engine.Server(0, 1, need // 2)
    try:
        t, _ = srv.submit(g, "msp")
        with pytest.raises(engine.BitrussError) as ei:
            srv.wait(t)
        assert ei.value.code == "BT_ERR_DEVICE_MEMORY"
    finally:
        srv.close()


@pytest.mark.gpu
def test_wait_timeout_keeps_ticket(engine):
    from gpu_bitruss_gb300 import gen
    g = engine.Graph.from_edges(*gen.by_name("cl200k"))
    srv = engine.Server(0, 1, 0)
    try:
        t, out = srv.submit(g, "msp")
        try:
            srv.wait(t, timeout_ms=0.0)
            done_early = True
        except engine.BitrussError as e:
            assert e.code == "BT_ERR_TIMEOUT"
            done_early = False
        info = srv.wait(t)
        assert info["status"] == 0 and info["levels"] == int(out.max())
        assert done_early in (True, False)
    finally:
        srv.close()


@pytest.mark.gpu
@pytest.mark.parametrize("op", ["bfc", "ebfc", "msp"])
def test_admission_estimate_bounds_the_peak(engine, gpu_ctx, op):
    """bt_job_bytes is an upper bound of what a job allocates (single graphs
    and arenas), so the server's budget is never exceeded."""
    from gpu_bitruss_gb300 import gen
    cases = [[engine.Graph.from_edges(*gen.by_name(nm))] for nm in ("cl50k", "cl200k")]
    cases.append([engine.Graph.from_edges(u, v) for u, v in random_lists(20, 4)])
    for graphs in cases:
        est = gpu_ctx.job_bytes(graphs, op)
        ctx = engine.Context(0)  # fresh: nothing resident before the job
        try:
            if len(graphs) == 1:
                ctx.upload(graphs[0])
                {"bfc": ctx.bfc, "ebfc": ctx.ebfc, "msp": ctx.msp}[op]()
            elif op == "msp":
                ctx.msp_batch(graphs)
            else:
                ctx.ebfc_batch(graphs)
            peak = ctx.memory_peak()
        finally:
            ctx.close()
        assert 0 < peak <= est, (op, peak, est)
