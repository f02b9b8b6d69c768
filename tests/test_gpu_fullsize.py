"""Config 2 at full size (Chung-Lu, 20M edges), against facts the oracle
computed (tests/golden/make_facts.py): butterfly count, largest support and
the digest of all 20M supports, bit for bit; size-independent properties of
the decomposition; and -- when the oracle's full decomposition is recorded in
tests/golden/cl20m.json -- the digest of the msp result itself."""

import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def test_cl20m_counts_and_decomposition(engine, gpu_ctx):
    from gpu_bitruss_gb300 import gen
    with open(os.path.join(GOLDEN, "cl20m.json")) as f:
        want = json.load(f)
    u, v = gen.by_name("cl20m")
    assert gen.digest(u, v) == want["edge_digest"]
    g = engine.Graph.from_edges(u, v)
    assert g.m == want["m"]
    gpu_ctx.upload(g)
    assert gpu_ctx.bfc() == want["count"]
    sup, count, sup_max = gpu_ctx.ebfc()
    assert count == want["count"] and sup_max == want["support_max"]
    assert int(sup.sum(dtype=np.uint64)) == 4 * want["count"]
    assert hashlib.sha256(sup.astype("<u8").tobytes()).hexdigest() == want["sup_sha256"]
    b, levels = gpu_ctx.msp()
    assert levels == int(b.max())
    assert bool((b.astype(np.uint64) <= sup).all())
    assert bool(((b == 0) == (sup == 0)).all())
    if "msp_sha256" in want:
        assert hashlib.sha256(b.astype("<u4").tobytes()).hexdigest() == want["msp_sha256"]
        assert levels == want["levels"]
    if "subrounds" in want:
        assert gpu_ctx.stats()[1] == want["subrounds"]
