"""Host-side engine code that needs no GPU: the CSR converter, .bin I/O,
error statuses, the C-ABI exports and the coh front end."""

import hashlib
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN_CASES, ROOT, load_golden


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_converter_matches_reference_bin(engine, tmp_path, name):
    gd = load_golden(name)
    g = engine.Graph.from_edges(gd["u"], gd["v"])
    p = str(tmp_path / "g.bin")
    g.to_bin(p)
    assert hashlib.sha256(open(p, "rb").read()).hexdigest() == str(gd["bin_sha256"])
    g2 = engine.Graph.from_bin(p)
    for k in ("offsets", "neighbors", "degrees", "edges", "edge_ids"):
        np.testing.assert_array_equal(getattr(g2, k), getattr(g, k))
    assert (g2.u_num, g2.l_num, g2.m) == (g.u_num, g.l_num, g.m)


def test_text_parsing_matches_edges(engine, tmp_path):
    gd = load_golden("er_small2")
    p = tmp_path / "g.txt"
    with open(p, "w") as f:
        f.write("% bip unweighted\n% 500 40 30\n")
        for i, (a, b) in enumerate(zip(gd["u"].tolist(), gd["v"].tolist())):
            # KONECT files may carry extra columns; blank lines are skipped
            f.write(f"{a} {b} 1 {i}\n" if i % 3 == 0 else f"{a}\t{b}\r\n")
            if i == 10:
                f.write("\n")
    g = engine.Graph.from_text(str(p))
    p2 = str(tmp_path / "g.bin")
    g.to_bin(p2)
    assert hashlib.sha256(open(p2, "rb").read()).hexdigest() == str(gd["bin_sha256"])


def test_duplicate_lines_are_kept_like_the_reference(engine, oracle_mod):
    u = np.array([0, 0, 1, 0, 1], np.uint32)
    v = np.array([0, 1, 0, 0, 1], np.uint32)
    g = engine.Graph.from_edges(u, v)
    o = oracle_mod.build_csr(u, v)
    assert g.m == 5
    for k in ("offsets", "neighbors", "degrees", "edges", "edge_ids"):
        np.testing.assert_array_equal(getattr(g, k), o[k])


@pytest.mark.parametrize("name", ["hub500k", "cl200k"])
def test_host_csr_equals_the_oracle_on_large_graphs(engine, oracle_mod, name):
    """The engine's text-order CSR (process_graph numbering, reference edge
    ids) equals the oracle's array for array on a hub-skewed graph (rows up to
    ~10^4 long) and a power-law graph."""
    from gpu_bitruss_gb300 import gen
    u, v = gen.by_name(name)
    g = engine.Graph.from_edges(u, v)
    o = oracle_mod.build_csr(u, v)
    assert (g.u_num, g.l_num, g.n, g.m) == (o["u_num"], o["l_num"], o["n"], o["m"])
    for key in ("offsets", "degrees", "neighbors", "edges", "edge_ids"):
        np.testing.assert_array_equal(getattr(g, key), o[key], err_msg=key)


def test_empty_graph(engine):
    g = engine.Graph.from_edges(np.zeros(0, np.uint32), np.zeros(0, np.uint32))
    assert (g.n, g.m) == (0, 0)


def test_id_limit(engine):
    with pytest.raises(engine.BitrussError) as ei:
        engine.Graph.from_edges(np.array([99999999], np.uint32), np.array([0], np.uint32))
    assert ei.value.code == "BT_ERR_INVALID"


def test_bad_text(engine, tmp_path):
    p = tmp_path / "bad.txt"
    p.write_text("1 2\n3\n")
    with pytest.raises(engine.BitrussError) as ei:
        engine.Graph.from_text(str(p))
    assert ei.value.code == "BT_ERR_FORMAT"
    with pytest.raises(engine.BitrussError) as ei:
        engine.Graph.from_text(str(tmp_path / "missing.txt"))
    assert ei.value.code == "BT_ERR_IO"


def test_bad_bin(engine, tmp_path):
    gd = load_golden("er_small1")
    g = engine.Graph.from_edges(gd["u"], gd["v"])
    p = str(tmp_path / "g.bin")
    g.to_bin(p)
    raw = open(p, "rb").read()
    # truncated
    open(p, "wb").write(raw[:-4])
    with pytest.raises(engine.BitrussError) as ei:
        engine.Graph.from_bin(p)
    assert ei.value.code == "BT_ERR_FORMAT"
    # header shorter than 5 words
    open(p, "wb").write(raw[:12])
    with pytest.raises(engine.BitrussError) as ei:
        engine.Graph.from_bin(p)
    assert ei.value.code == "BT_ERR_FORMAT"
    # neighbour id out of range
    arr = np.frombuffer(raw, dtype="<u4").copy()
    arr[5] = 10 ** 6
    open(p, "wb").write(arr.tobytes())
    with pytest.raises(engine.BitrussError) as ei:
        engine.Graph.from_bin(p)
    assert ei.value.code == "BT_ERR_FORMAT"


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "bitruss.h")).read()
    return sorted(set(re.findall(r"\b(bt_[a-z_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(engine):
    syms = declared_symbols()
    assert len(syms) >= 20
    lib = engine.load()
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    assert sorted(engine.SYMBOLS) == syms


def test_status_strings(engine):
    lib = engine.load()
    for code in engine.STATUS:
        assert lib.bt_status_string(code)


def test_no_device_is_an_error_not_a_fallback(engine):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(engine.BitrussError) as ei:
        engine.Context(0)
    assert ei.value.code == "BT_ERR_NO_DEVICE"


def test_coh_converts_like_the_reference(engine, tmp_path):
    gd = load_golden("aw")
    txt = tmp_path / "aw.graph"
    txt.write_text("".join(f"{a} {b}\n" for a, b in zip(gd["u"].tolist(), gd["v"].tolist())))
    out = tmp_path / "aw.bin"
    r = subprocess.run([engine.COH_PATH, "--graph", str(txt), "--bin", str(out)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert hashlib.sha256(out.read_bytes()).hexdigest() == str(gd["bin_sha256"])
    r = subprocess.run([engine.COH_PATH, "--bogus"], capture_output=True, text=True)
    assert r.returncode != 0 and "Unknown argument" in r.stdout
