"""CUDA engine vs the reference (golden vectors) and the oracle, through the
C ABI.  Integer outputs: bit-exact."""

import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_counts_and_supports(engine, gpu_ctx, name):
    gd = load_golden(name)
    g = engine.Graph.from_edges(gd["u"], gd["v"])
    gpu_ctx.upload(g)
    assert gpu_ctx.bfc() == int(gd["bfc"])
    sup, cnt, mx = gpu_ctx.ebfc()
    np.testing.assert_array_equal(sup, gd["ebfc"])
    assert cnt == int(gd["count"])
    assert mx == (int(gd["ebfc"].max()) if g.m else 0)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_msp_matches_reference(engine, gpu_ctx, name):
    gd = load_golden(name)
    g = engine.Graph.from_edges(gd["u"], gd["v"])
    gpu_ctx.upload(g)
    b, levels = gpu_ctx.msp()
    np.testing.assert_array_equal(b.astype(np.uint64), gd["msp"])
    assert levels == int(gd["levels"])
    # second call on the same resident graph gives the same answer
    b2, levels2 = gpu_ctx.msp()
    np.testing.assert_array_equal(b2, b)
    assert levels2 == levels


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_hidx_and_exact_msp_match_reference_hidx(engine, gpu_ctx, name):
    gd = load_golden(name)
    g = engine.Graph.from_edges(gd["u"], gd["v"])
    gpu_ctx.upload(g)
    h, rounds = gpu_ctx.hidx()
    np.testing.assert_array_equal(h.astype(np.uint64), gd["hidx"])
    assert rounds >= 1
    x, _ = gpu_ctx.msp(exact=True)
    np.testing.assert_array_equal(x.astype(np.uint64), gd["hidx"])


def test_reference_api_mirror(engine):
    gd = load_golden("er_config1")
    g = engine.Graph.from_edges(gd["u"], gd["v"])
    assert engine.bfc_vpp(g) == int(gd["count"])
    np.testing.assert_array_equal(engine.bfc_evpp(g), gd["ebfc"])
    np.testing.assert_array_equal(engine.bitruss_msp(g).astype(np.uint64), gd["msp"])
    assert g.levels == int(gd["levels"])
    np.testing.assert_array_equal(engine.g_bitruss_hindex(g).astype(np.uint64), gd["hidx"])


def _k(a, b):
    u = np.repeat(np.arange(a, dtype=np.uint32), b)
    v = np.tile(np.arange(b, dtype=np.uint32), a)
    return u, v


@pytest.mark.parametrize("shape", [(1, 1), (1, 9), (9, 1), (2, 2), (5, 7), (40, 3), (64, 64)])
def test_complete_bipartite(engine, gpu_ctx, oracle_mod, shape):
    a, b = shape
    u, v = _k(a, b)
    g = engine.Graph.from_edges(u, v)
    gpu_ctx.upload(g)
    sup, cnt, _ = gpu_ctx.ebfc()
    assert cnt == (a * (a - 1) // 2) * (b * (b - 1) // 2)
    assert np.all(sup == (a - 1) * (b - 1))
    res, levels = gpu_ctx.msp()
    assert np.all(res == (a - 1) * (b - 1))
    assert levels == (a - 1) * (b - 1)


def test_empty_and_single_edge(engine, gpu_ctx):
    for u, v in ((np.zeros(0, np.uint32), np.zeros(0, np.uint32)),
                 (np.array([3], np.uint32), np.array([4], np.uint32))):
        g = engine.Graph.from_edges(u, v)
        gpu_ctx.upload(g)
        assert gpu_ctx.bfc() == 0
        sup, cnt, mx = gpu_ctx.ebfc()
        assert cnt == 0 and mx == 0 and np.all(sup == 0)
        b, levels = gpu_ctx.msp()
        assert levels == 0 and np.all(b == 0)
        h, _ = gpu_ctx.hidx()
        assert np.all(h == 0)


@pytest.mark.parametrize("seed", range(8))
def test_random_small_vs_oracle(engine, gpu_ctx, oracle_mod, seed):
    from gpu_bitruss_gb300 import gen
    rng = np.random.default_rng(seed)
    nu, nv = int(rng.integers(5, 60)), int(rng.integers(5, 60))
    m = int(rng.integers(1, nu * nv // 2 + 2))
    u, v = gen.er(nu, nv, m, seed=1000 + seed)
    g = engine.Graph.from_edges(u, v)
    o = oracle_mod.build_csr(u, v)
    sup, cnt = oracle_mod.ebfc(o, 2)
    ref, levels, _ = oracle_mod.msp(o, 2, oracle_mod.MSP_REF, sup)
    h, _ = oracle_mod.hidx(o, 2, sup)
    gpu_ctx.upload(g)
    gs, gc, _ = gpu_ctx.ebfc()
    np.testing.assert_array_equal(gs, sup)
    b, lv = gpu_ctx.msp()
    np.testing.assert_array_equal(b.astype(np.uint64), ref)
    assert lv == levels
    x, _ = gpu_ctx.msp(exact=True)
    np.testing.assert_array_equal(x.astype(np.uint64), h)


@pytest.mark.parametrize("name", ["cl50k", "cl200k"])
def test_power_law_vs_oracle(engine, gpu_ctx, oracle_mod, name):
    from gpu_bitruss_gb300 import gen
    u, v = gen.by_name(name)
    g = engine.Graph.from_edges(u, v)
    o = oracle_mod.build_csr(u, v)
    sup, cnt = oracle_mod.ebfc(o, 0)
    ref, levels, _ = oracle_mod.msp(o, 0, oracle_mod.MSP_TABLE, sup)
    gpu_ctx.upload(g)
    gs, gc, _ = gpu_ctx.ebfc()
    np.testing.assert_array_equal(gs, sup)
    assert gc == cnt
    b, lv = gpu_ctx.msp()
    np.testing.assert_array_equal(b.astype(np.uint64), ref)
    assert lv == levels


@pytest.mark.parametrize("name", ["aw", "er_config1", "er_small2", "er_small3", "cl5k", "cl20k"])
def test_hidx_rounds_match_the_oracle(engine, gpu_ctx, oracle_mod, name):
    """Rounds recompute only edges next to a change, yet take exactly as many
    rounds as the full synchronous iteration (the reference's count)."""
    gd = load_golden(name)
    g = engine.Graph.from_edges(gd["u"], gd["v"])
    gpu_ctx.upload(g)
    h, rounds = gpu_ctx.hidx()
    np.testing.assert_array_equal(h.astype(np.uint64), gd["hidx"])
    want, want_rounds = oracle_mod.hidx(oracle_mod.build_csr(gd["u"], gd["v"]), 1)
    assert rounds == want_rounds
    st = gpu_ctx.stats()
    recomputed = st[18]
    assert g.m <= recomputed <= rounds * g.m
    assert st[19] == 0  # started from the supports, as the reference does


@pytest.mark.parametrize("name", ["aw", "er_config1", "er_small2", "er_small3", "cl5k", "cl20k", "sparse"])
def test_hidx_from_the_exact_peel_reaches_the_same_fixpoint(engine, gpu_ctx, name, monkeypatch):
    """Started from the exact peel's values instead of the supports, the
    h-index iteration ends at the same per-edge values (the reference's
    hidx), after one round that changes nothing."""
    gd = load_golden(name)
    g = engine.Graph.from_edges(gd["u"], gd["v"])
    gpu_ctx.upload(g)
    monkeypatch.setenv("BT_HIDX_START", "peel")
    h, rounds = gpu_ctx.hidx()
    np.testing.assert_array_equal(h.astype(np.uint64), gd["hidx"])
    st = gpu_ctx.stats()
    assert rounds == 1 and st[19] == 1
    assert st[18] == g.m
    monkeypatch.setenv("BT_HIDX_START", "support")
    h2, rounds2 = gpu_ctx.hidx()
    np.testing.assert_array_equal(h2, h)
    assert gpu_ctx.stats()[19] == 0 and rounds2 >= 1


@pytest.mark.parametrize("name", ["aw", "er_config1", "er_small3", "cl5k", "cl20k"])
def test_msp_with_64bit_working_supports(engine, gpu_ctx, name, monkeypatch):
    """Graphs whose supports all fit 32 bits peel with 32-bit working supports;
    the 64-bit path (supports above 2^32) gives the same results."""
    gd = load_golden(name)
    g = engine.Graph.from_edges(gd["u"], gd["v"])
    gpu_ctx.upload(g)
    monkeypatch.setenv("BT_MSP_WIDE", "1")
    b, levels = gpu_ctx.msp()
    np.testing.assert_array_equal(b.astype(np.uint64), gd["msp"])
    assert levels == int(gd["levels"])
    x, _ = gpu_ctx.msp(exact=True)
    np.testing.assert_array_equal(x.astype(np.uint64), gd["hidx"])


def test_kernel_launch_count(engine, gpu_ctx):
    """A bt_msp call on a resident graph launches the library's own kernels
    k_count, k_msp_init, k_two_hop and the persistent k_msp: four launches,
    whatever the number of levels and sub-rounds."""
    gd = load_golden("cl20k")
    g = engine.Graph.from_edges(gd["u"], gd["v"])
    gpu_ctx.upload(g)
    before = engine.kernel_launches()
    gpu_ctx.msp()
    assert engine.kernel_launches() - before == 4
