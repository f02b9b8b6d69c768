"""Failure handling on the GPU, without faulting it: a device-side wait that
runs out, an allocation refused by the memory budget, the coh front end and
the C++ drop-in header.

The waits in the peeling kernel (its grid barrier) are bounded.  With a 1 us
limit some CTA is sure to wait longer for the others; the kernel must then
report BT_ERR_TIMEOUT, return, and leave the context usable.
"""

import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_golden

pytestmark = pytest.mark.gpu


def test_barrier_wait_limit_reports_timeout_and_context_survives(engine, gpu_ctx):
    gd = load_golden("cl20k")
    g = engine.Graph.from_edges(gd["u"], gd["v"])
    gpu_ctx.upload(g)
    old = os.environ.get("BT_WAIT_LIMIT_US")
    os.environ["BT_WAIT_LIMIT_US"] = "1"
    try:
        with pytest.raises(engine.BitrussError) as ei:
            gpu_ctx.msp()
        assert ei.value.code == "BT_ERR_TIMEOUT"
    finally:
        if old is None:
            del os.environ["BT_WAIT_LIMIT_US"]
        else:
            os.environ["BT_WAIT_LIMIT_US"] = old
    b, levels = gpu_ctx.msp()
    np.testing.assert_array_equal(b.astype(np.uint64), gd["msp"])
    assert levels == int(gd["levels"])


def test_memory_budget_refuses_and_recovers(engine):
    gd = load_golden("cl20k")
    g = engine.Graph.from_edges(gd["u"], gd["v"])
    ctx = engine.Context(0)
    try:
        ctx.set_budget(1 << 16)
        with pytest.raises(engine.BitrussError) as ei:
            ctx.upload(g)
        assert ei.value.code == "BT_ERR_DEVICE_MEMORY"
        assert ctx.memory_used() <= (1 << 16)
        ctx.set_budget(0)
        ctx.upload(g)
        used = ctx.memory_used()
        assert used > 0
        # msp needs working memory beyond the resident graph
        ctx.set_budget(used + (1 << 16))
        with pytest.raises(engine.BitrussError) as ei:
            ctx.msp()
        assert ei.value.code == "BT_ERR_DEVICE_MEMORY"
        ctx.set_budget(0)
        b, _ = ctx.msp()
        np.testing.assert_array_equal(b.astype(np.uint64), gd["msp"])
    finally:
        ctx.close()


def test_no_graph_is_a_state_error(engine):
    ctx = engine.Context(0)
    try:
        with pytest.raises(engine.BitrussError) as ei:
            ctx.bfc()
        assert ei.value.code == "BT_ERR_STATE"
    finally:
        ctx.close()


def test_coh_gpu_msp_end_to_end(engine, tmp_path):
    gd = load_golden("er_config1")
    txt = tmp_path / "g.txt"
    txt.write_text("".join(f"{a} {b}\n" for a, b in zip(gd["u"].tolist(), gd["v"].tolist())))
    binf = tmp_path / "g.bin"
    out = tmp_path / "res.txt"
    r = subprocess.run([engine.COH_PATH, "--graph", str(txt), "--bin", str(binf)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    for algo, key in (("msp", "msp"), ("hidx", "hidx")):
        r = subprocess.run([engine.COH_PATH, "--graph", str(binf), "--gpu", "--algo", algo, "--out", str(out)],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        vals = np.loadtxt(out, dtype=np.uint64)[:, 2]
        np.testing.assert_array_equal(vals, gd[key])
    assert f"bitruss msp with {int(gd['levels'])} levels" in subprocess.run(
        [engine.COH_PATH, "--graph", str(binf), "--gpu", "--algo", "msp"], capture_output=True, text=True).stdout
    r = subprocess.run([engine.COH_PATH, "--graph", str(binf), "--gpu", "--algo", "bfc"], capture_output=True, text=True)
    assert f"btf number: {int(gd['bfc'])}" in r.stdout


def test_cpp_header_graph_loop_uploads_every_graph(engine, tmp_path):
    """bitruss.hpp in a loop over files, one stack Graph per iteration (the
    same address each time): each file's results equal its own goldens."""
    src = os.path.join(ROOT, "tests", "cpp", "hpp_graph_loop.cpp")
    exe = tmp_path / "hpp_graph_loop"
    pkg = os.path.dirname(engine.LIB_PATH)
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), src, "-o", str(exe),
                        "-L", pkg, "-lbitruss", f"-Wl,-rpath,{pkg}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    names = ["aw", "er_config1", "er_small0", "aw", "er_config1"]
    files = []
    for i, name in enumerate(names):
        gd = load_golden(name)
        p = tmp_path / f"g{i}.txt"
        p.write_text("".join(f"{a} {b}\n" for a, b in zip(gd["u"].tolist(), gd["v"].tolist())))
        files.append(str(p))
    r = subprocess.run([str(exe)] + files, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = r.stdout.strip().splitlines()
    assert len(lines) == len(names)
    for name, line in zip(names, lines):
        gd = load_golden(name)
        vals = np.array(line.split(), dtype=np.uint64)
        assert vals[0] == gd["bfc"], name
        assert vals[1] == gd["levels"], name
        np.testing.assert_array_equal(vals[2:], gd["msp"], err_msg=name)
