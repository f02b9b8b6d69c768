"""Generate the golden fixtures from the reference's own CPU code.

Run here (where the reference sources are present):

    python tests/golden/make_golden.py

It builds oracle/_ref/libref.so from the reference sources (oracle/Makefile,
target "ref"), then for each case writes the edge list in file order to a
"u v" text file, converts it with the reference's Graph(text, true) +
graph_to_bin, and runs the reference CPU algorithms with one thread (the
reference's msp and hidx race with more than one thread: scan_edge writes a
std::vector<bool> from several threads, cpu_bitruss.cpp:285-299, and
c_bitruss_hindex re-arms `converge` inside the parallel region,
cpu_bitruss.cpp:243-244).  Results go to tests/golden/<case>.npz:

    u, v            uint32 edge list in file order
    ebfc            uint64 per-edge support     (cpu_bfc.cpp:24-122)
    count           butterfly total (ebfc log)  (cpu_bfc.cpp:120)
    bfc             butterfly total (bfc log)   (cpu_bfc.cpp:201)
    hidx            uint64 bitruss numbers      (cpu_bitruss.cpp:227-266)
    msp             uint64 bitruss numbers      (cpu_bitruss.cpp:563-624)
    levels          msp level count (log)       (cpu_bitruss.cpp:621)
    bin_sha256      sha256 of the reference .bin
"""

from __future__ import annotations

import hashlib
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from gpu_bitruss_gb300 import gen  # noqa: E402
from oracle import oracle as O  # noqa: E402

AW = os.path.join(O.REF_ROOT, "data", "aw.graph")  # the reference's sample graph


def cases():
    # the reference's own sample graph (data/aw.graph)
    uv = np.loadtxt(AW, dtype=np.uint32).reshape(-1, 2)
    yield "aw", uv[:, 0].copy(), uv[:, 1].copy()
    # config 1: ER 2,000 x 3,000, 20,000 unique edges, seed 1
    yield "er_config1", *gen.er()
    # small dense random graphs: many sub-rounds, msp != hidx on some
    for i, (nu, nv, m) in enumerate([(12, 15, 60), (30, 40, 300), (40, 30, 500),
                                     (60, 80, 1500), (200, 150, 3000)]):
        yield f"er_small{i}", *gen.er(nu, nv, m, seed=100 + i)
    # small power-law graphs (hubs)
    yield "cl5k", *gen.by_name("cl5k")
    yield "cl20k", *gen.by_name("cl20k")
    # sparse graph with zero-support edges and isolated stars
    yield "sparse", *gen.er(500, 500, 600, seed=7)


def main():
    O.build(ref=True)
    with tempfile.TemporaryDirectory() as d:
        for name, u, v in cases():
            txt = os.path.join(d, name + ".graph")
            b = os.path.join(d, name + ".bin")
            gen.to_text(txt, u, v)
            O.ref_convert(txt, b)
            rb = O.read_bin(b)
            m = rb["m"]
            ebfc, log = O.ref_run(b, "ebfc", 1, m)
            count = O.ref_log_count(log)
            _, log_b = O.ref_run(b, "bfc", 1, m)
            bfc = O.ref_log_count(log_b)
            hidx, _ = O.ref_run(b, "hidx", 1, m)
            msp, log_m = O.ref_run(b, "msp", 1, m)
            levels = O.ref_log_levels(log_m)
            sha = hashlib.sha256(open(b, "rb").read()).hexdigest()
            np.savez_compressed(
                os.path.join(HERE, name + ".npz"), u=u, v=v,
                ebfc=ebfc.astype(np.uint64), count=np.uint64(count), bfc=np.uint64(bfc),
                hidx=hidx.astype(np.uint64), msp=msp.astype(np.uint64),
                levels=np.uint64(levels), bin_sha256=np.array(sha))
            print(f"{name}: m={m} count={count} levels={levels} "
                  f"msp!=hidx={(msp != hidx).sum()} max_sup={ebfc.max() if m else 0}")


if __name__ == "__main__":
    main()
