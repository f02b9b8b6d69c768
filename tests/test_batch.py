"""Batched arenas: many graphs packed into one disjoint-union CSR.

CPU tests check the packing against the reference numbering of the
concatenated edge lists, and check on the oracle (and on the reference's own
CPU code where it is built) that peeling the union gives every graph its
single-graph result.  GPU tests run the batched C-ABI calls against the
golden vectors and the oracle, bit for bit.
"""

import os
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden

BATCH_CASES = [c for c in GOLDEN_CASES if c != "cl20k"]


def concat_edges(lists):
    """Concatenate (u, v) edge lists with disjoint raw ids, in list order."""
    us, vs, uo, vo = [], [], 0, 0
    for u, v in lists:
        u = np.asarray(u, np.uint64)
        v = np.asarray(v, np.uint64)
        us.append(u + uo)
        vs.append(v + vo)
        if u.size:
            uo += int(u.max()) + 1
            vo += int(v.max()) + 1
    cat = lambda a: np.concatenate(a).astype(np.uint32) if a else np.zeros(0, np.uint32)
    return cat(us), cat(vs)


def golden_lists(names):
    gds = [load_golden(n) for n in names]
    return gds, [(gd["u"], gd["v"]) for gd in gds]


def random_lists(count, seed):
    from gpu_bitruss_gb300 import gen
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        kind = rng.integers(0, 3)
        if kind == 0:
            nu, nv = int(rng.integers(4, 60)), int(rng.integers(4, 60))
            m = int(rng.integers(1, min(nu * nv, 600) + 1))
            out.append(gen.er(nu, nv, m, seed=1000 + i))
        elif kind == 1:
            m = int(rng.integers(200, 3000))
            out.append(gen.chung_lu(max(m // 8, 16), max(m // 10, 16), m, 2.3, 2.3, 40, 40, seed=2000 + i))
        else:
            out.append((np.zeros(0, np.uint32), np.zeros(0, np.uint32)))
    return out


# ---------------------------------------------------------------------------
# CPU
# ---------------------------------------------------------------------------

def test_pack_equals_reference_numbering_of_concatenation(engine):
    _, lists = golden_lists(BATCH_CASES)
    lists = lists + random_lists(12, 5)
    graphs = [engine.Graph.from_edges(u, v) for u, v in lists]
    arena, base = engine.pack(graphs)
    whole = engine.Graph.from_edges(*concat_edges(lists))
    assert (arena.u_num, arena.l_num, arena.n, arena.m) == (whole.u_num, whole.l_num, whole.n, whole.m)
    for k in ("offsets", "degrees", "neighbors", "edges", "edge_ids"):
        np.testing.assert_array_equal(getattr(arena, k), getattr(whole, k), err_msg=k)
    np.testing.assert_array_equal(np.diff(base.astype(np.int64)), [g.m for g in graphs])


def test_pack_empty_and_single(engine):
    arena, base = engine.pack([])
    assert arena.m == 0 and arena.n == 0 and list(base) == [0]
    gd = load_golden("aw")
    g = engine.Graph.from_edges(gd["u"], gd["v"])
    arena, base = engine.pack([g])
    for k in ("offsets", "degrees", "neighbors", "edges", "edge_ids"):
        np.testing.assert_array_equal(getattr(arena, k), getattr(g, k))


def test_union_peel_equals_per_graph_on_oracle(oracle_mod):
    """The disjoint-union argument, on the oracle: msp, exact msp, supports."""
    O = oracle_mod
    gds, lists = golden_lists(BATCH_CASES)
    lists = lists + random_lists(10, 7)
    whole = O.build_csr(*concat_edges(lists))
    sup, cnt = O.ebfc(whole, 1)
    res, levels, _ = O.msp(whole, 1, O.MSP_REF, sup)
    ex, _, _ = O.msp(whole, 1, O.MSP_EXACT, sup)
    e0, total_count, max_level = 0, 0, 0
    for i, (u, v) in enumerate(lists):
        g = O.build_csr(u, v)
        m = g["m"]
        s1, c1 = O.ebfc(g, 1)
        r1, l1, _ = O.msp(g, 1, O.MSP_REF, s1)
        x1, _, _ = O.msp(g, 1, O.MSP_EXACT, s1)
        np.testing.assert_array_equal(sup[e0:e0 + m], s1)
        np.testing.assert_array_equal(res[e0:e0 + m], r1)
        np.testing.assert_array_equal(ex[e0:e0 + m], x1)
        assert l1 == (int(r1.max()) if m else 0), "levels = largest bitruss number"
        if i < len(gds):
            np.testing.assert_array_equal(r1, gds[i]["msp"])
        total_count += c1
        max_level = max(max_level, l1)
        e0 += m
    assert cnt == total_count
    assert levels == max_level


def test_union_peel_equals_per_graph_on_reference(oracle_mod):
    """The same on the reference's own CPU code (built from its sources here)."""
    O = oracle_mod
    if not O.ref_available():
        pytest.skip("reference CPU code not built on this host")
    gds, lists = golden_lists(["aw", "er_config1", "er_small1", "er_small3", "sparse"])
    u, v = concat_edges(lists)
    with tempfile.TemporaryDirectory() as d:
        txt, binp = os.path.join(d, "g.txt"), os.path.join(d, "g.bin")
        with open(txt, "w") as f:
            for a, b in zip(u.tolist(), v.tolist()):
                f.write(f"{a} {b}\n")
        O.ref_convert(txt, binp)
        m = int(u.size)
        out, log = O.ref_run(binp, "msp", 1, m)
    e0 = 0
    for gd in gds:
        k = gd["u"].size
        np.testing.assert_array_equal(np.asarray(out[e0:e0 + k], np.uint64), gd["msp"])
        e0 += k


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------

@pytest.mark.gpu
@pytest.mark.parametrize("arena_edges", [1 << 28, 3000])
def test_msp_batch_matches_goldens(engine, gpu_ctx, arena_edges):
    gds, lists = golden_lists(GOLDEN_CASES)
    graphs = [engine.Graph.from_edges(u, v) for u, v in lists]
    gpu_ctx.set_arena_edges(arena_edges)
    try:
        res, levels = gpu_ctx.msp_batch(graphs)
        for gd, r, lv in zip(gds, res, levels):
            np.testing.assert_array_equal(r.astype(np.uint64), gd["msp"])
            assert int(lv) == int(gd["levels"])
        arenas = gpu_ctx.stats()[7]
        assert arenas == 1 if arena_edges > 100000 else arenas > 1
        ex, _ = gpu_ctx.msp_batch(graphs, exact=True)
        for gd, x in zip(gds, ex):
            np.testing.assert_array_equal(x.astype(np.uint64), gd["hidx"])
        sup, counts = gpu_ctx.ebfc_batch(graphs)
        for gd, s, c in zip(gds, sup, counts):
            np.testing.assert_array_equal(s, gd["ebfc"])
            assert int(c) == int(gd["count"])
    finally:
        gpu_ctx.set_arena_edges(1 << 28)


@pytest.mark.gpu
def test_msp_batch_random_vs_oracle(engine, gpu_ctx, oracle_mod):
    O = oracle_mod
    lists = random_lists(60, 11)
    graphs = [engine.Graph.from_edges(u, v) for u, v in lists]
    res, levels = gpu_ctx.msp_batch(graphs)
    for (u, v), r, lv in zip(lists, res, levels):
        g = O.build_csr(u, v)
        want, wl, _ = O.msp(g, 0, O.MSP_REF)
        np.testing.assert_array_equal(r.astype(np.uint64), want)
        assert int(lv) == wl


@pytest.mark.gpu
def test_peel_on_a_share_of_the_sms(engine, gpu_ctx):
    """The peeling kernel on fewer CTAs than SMs gives the same results."""
    gd = load_golden("cl20k")
    g = engine.Graph.from_edges(gd["u"], gd["v"])
    gpu_ctx.upload(g)
    try:
        for ctas in (1, 7, 38, 76, 100000):
            gpu_ctx.set_peel_ctas(ctas)
            b, lv = gpu_ctx.msp()
            np.testing.assert_array_equal(b.astype(np.uint64), gd["msp"])
            assert lv == int(gd["levels"])
    finally:
        gpu_ctx.set_peel_ctas(0)


@pytest.mark.gpu
def test_msp_batch_empty(engine, gpu_ctx):
    res, levels = gpu_ctx.msp_batch([])
    assert res == [] and len(levels) == 0
    e = (np.zeros(0, np.uint32), np.zeros(0, np.uint32))
    res, levels = gpu_ctx.msp_batch([engine.Graph.from_edges(*e)] * 3)
    assert all(r.size == 0 for r in res) and list(levels) == [0, 0, 0]


@pytest.mark.gpu
def test_schedules_do_not_change_results(engine, gpu_ctx):
    gd = load_golden("cl20k")
    g = engine.Graph.from_edges(gd["u"], gd["v"])
    gpu_ctx.upload(g)
    try:
        for sched in [(512, 1, 64), (8192, 4, 512), (1024, 3, 256), (4096, 1, 1)]:
            gpu_ctx.set_msp_schedule(*sched)
            assert gpu_ctx.msp_schedule() == sched
            b, lv = gpu_ctx.msp()
            np.testing.assert_array_equal(b.astype(np.uint64), gd["msp"])
            assert lv == int(gd["levels"])
        gpu_ctx.set_msp_schedule(0, 0, 0)
        best, ms = gpu_ctx.autotune()
        assert ms > 0 and gpu_ctx.msp_schedule() == best
        b, _ = gpu_ctx.msp()
        np.testing.assert_array_equal(b.astype(np.uint64), gd["msp"])
    finally:
        gpu_ctx.set_msp_schedule(0, 0, 0)


def test_schedule_arguments_are_checked(engine):
    import gpu_bitruss_gb300 as bt
    L = bt.load()
    # a null context is rejected before any device work
    assert L.bt_ctx_set_msp_schedule(None, 0, 0, 0) == 1
    assert L.bt_ctx_set_arena_edges(None, 10) == 1
    assert L.bt_msp_batch(None, None, 0, 0, None, None) == 1


@pytest.mark.gpu
def test_msp_batch_on_the_batch_distribution_vs_oracle(engine, gpu_ctx, oracle_mod):
    """Graphs of the 4,096-graph batch itself (m log-uniform in [1e3, 2e6],
    Chung-Lu gamma 2.3, seed 4+i): the first ten of them small enough for the
    CPU oracle, packed in one arena; every graph's bitruss numbers and level
    count equal the oracle's."""
    from gpu_bitruss_gb300 import gen
    O = oracle_mod
    sizes = gen.batch_sizes()
    picks = [i for i in range(200) if sizes[0][i] <= 150_000][:10]
    lists = [gen.batch_graph(i, sizes=sizes) for i in picks]
    graphs = [engine.Graph.from_edges(u, v) for u, v in lists]
    res, levels = gpu_ctx.msp_batch(graphs)
    for (u, v), r, lv in zip(lists, res, levels):
        g = O.build_csr(u, v)
        want, wl, _ = O.msp(g, 0, O.MSP_TABLE)
        np.testing.assert_array_equal(r.astype(np.uint64), want)
        assert int(lv) == wl
