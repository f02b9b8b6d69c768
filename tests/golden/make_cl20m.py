"""Facts of config 2 (gen.by_name('cl20m'), 20M edges) computed by the oracle,
for tests/test_gpu_fullsize.py: butterfly count, largest support, the sha256
of the per-edge supports and, with --msp, of the msp bitruss numbers (the
full CPU decomposition takes hours).

    python tests/golden/make_cl20m.py [--msp] [--threads T]
"""

import argparse
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--msp", action="store_true")
    ap.add_argument("--threads", type=int, default=0)
    args = ap.parse_args()
    from gpu_bitruss_gb300 import gen
    from oracle import oracle as O
    O.build(ref=False)
    u, v = gen.by_name("cl20m")
    g = O.build_csr(u, v)
    path = os.path.join(HERE, "cl20m.json")
    out = json.load(open(path)) if os.path.exists(path) else {}
    out.update({"_what": "config 2 (gen.by_name('cl20m')): oracle results (oracle/bt_oracle.c)",
                "edge_digest": gen.digest(u, v), "m": int(g["m"])})
    t = time.time()
    sup, count = O.ebfc(g, args.threads)
    out.update({"count": int(count), "support_max": int(sup.max()),
                "sup_sha256": hashlib.sha256(sup.astype("<u8").tobytes()).hexdigest(),
                "ebfc_seconds": round(time.time() - t, 1)})
    if args.msp:
        t = time.time()
        res, levels, st = O.msp(g, args.threads, O.MSP_TABLE, sup)
        out.update({"levels": int(levels), "subrounds": int(st[1]),
                    "msp_sha256": hashlib.sha256(res.astype("<u4").tobytes()).hexdigest(),
                    "msp_seconds": round(time.time() - t, 1),
                    "msp_threads": args.threads or os.cpu_count()})
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
