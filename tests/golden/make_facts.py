"""Facts of a full-size workload computed by the oracle (oracle/bt_oracle.c),
for the full-size GPU tests and the bench's roofline: butterfly count,
largest support and the sha256 of the per-edge supports; with --msp the
sha256 of the msp bitruss numbers (the reference rule), the level and
sub-round counts and the algorithmic bytes of the reference's peeling walk;
with --exact the sha256 of the true bitruss numbers (the corrected rule, which
the h-index iteration and bt_msp_exact must equal).  The full CPU
decompositions take hours on large graphs.

    python tests/golden/make_facts.py [--workload cl20m] [--msp] [--exact] [--threads T]

Results go to tests/golden/<workload>.json (existing keys are kept).
"""

import argparse
import hashlib
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="cl20m")
    ap.add_argument("--msp", action="store_true")
    ap.add_argument("--exact", action="store_true")
    ap.add_argument("--threads", type=int, default=0)
    args = ap.parse_args()
    from gpu_bitruss_gb300 import gen
    from oracle import oracle as O
    O.build(ref=False)
    u, v = gen.by_name(args.workload)
    g = O.build_csr(u, v)
    path = os.path.join(HERE, f"{args.workload}.json")
    out = json.load(open(path)) if os.path.exists(path) else {}
    out.update({"_what": f"gen.by_name('{args.workload}'): oracle results (oracle/bt_oracle.c)",
                "edge_digest": gen.digest(u, v), "m": int(g["m"]), "n": int(g["n"])})
    threads = args.threads or os.cpu_count()
    t = time.time()
    sup, count = O.ebfc(g, args.threads)
    out.update({"count": int(count), "support_max": int(sup.max()) if g["m"] else 0,
                "sup_sha256": hashlib.sha256(sup.astype("<u8").tobytes()).hexdigest(),
                "ebfc_seconds": round(time.time() - t, 1)})
    if args.msp:
        t = time.time()
        res, levels, st = O.msp(g, args.threads, O.MSP_TABLE, sup)
        out.update({"levels": int(levels), "subrounds": int(st[1]),
                    "msp_sha256": hashlib.sha256(res.astype("<u4").tobytes()).hexdigest(),
                    "msp_seconds": round(time.time() - t, 1), "msp_threads": threads,
                    "oracle_msp_s": round(time.time() - t, 1), "oracle_threads": threads,
                    "msp_row_bytes": int(st[4]), "msp_butterflies_visited": int(st[5]),
                    "msp_decrements": int(st[6]), "msp_alg_bytes": int(st[7])})
    if args.exact:
        t = time.time()
        res, levels, st = O.msp(g, args.threads, O.MSP_TABLE_EXACT, sup)
        out.update({"exact_levels": int(levels), "exact_subrounds": int(st[1]),
                    "exact_sha256": hashlib.sha256(res.astype("<u4").tobytes()).hexdigest(),
                    "exact_seconds": round(time.time() - t, 1), "exact_threads": threads})
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
