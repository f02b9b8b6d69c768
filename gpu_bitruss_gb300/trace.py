"""Summarise a peeling-kernel trace (what bounds each msp sub-round).

Setting ``BT_MSP_TRACE=<path>`` makes ``bt_msp`` write one record per
sub-round: the sub-round's duration as seen by CTA 0 (plan to barrier exit),
its longest task, the row positions walked, the frontier size and the task
count.  Usage::

    BT_MSP_TRACE=trace.bin python bench.py --steps 1 --warmup 0 --no-cpu
    python -m gpu_bitruss_gb300.trace trace.bin
"""

from __future__ import annotations

import sys

import numpy as np

RECORD = np.dtype([("t_ns", "<u8"), ("max_task_ns", "<u8"), ("walked", "<u8"),
                   ("frontier", "<u4"), ("tasks", "<u4")])


def load(path: str) -> np.ndarray:
    """Sub-round records (the first two records are reserved)."""
    tr = np.fromfile(path, dtype=RECORD)[2:]
    return tr[tr["t_ns"] > 0]


def summary(tr: np.ndarray) -> str:
    out = []
    t = tr["t_ns"].astype(np.float64)
    mx = tr["max_task_ns"].astype(np.float64)
    w = tr["walked"].astype(np.float64)
    out.append(f"sub-rounds: {len(tr)}; sum of durations {t.sum() / 1e9:.2f} s; "
               f"sum of longest tasks {mx.sum() / 1e9:.2f} s; positions walked {w.sum():.4g}")
    p = np.percentile(t, [50, 90, 99]) / 1e3
    q = np.percentile(mx, [50, 90, 99]) / 1e3
    o = np.percentile(t - mx, [50, 90]) / 1e3
    out.append(f"duration us p50/p90/p99: {p[0]:.1f} / {p[1]:.1f} / {p[2]:.1f}")
    out.append(f"longest task us p50/p90/p99: {q[0]:.1f} / {q[1]:.1f} / {q[2]:.1f}")
    out.append(f"duration minus longest task us p50/p90: {o[0]:.1f} / {o[1]:.1f}")
    out.append("")
    out.append("| positions walked | sub-rounds | time s | mean us | mean longest task us | "
               "positions per us | mean frontier |")
    out.append("|---|---|---|---|---|---|---|")
    edges = [0, 1e4, 1e5, 1e6, 1e7, 1e8, 1e18]
    for lo, hi in zip(edges[:-1], edges[1:]):
        sel = (w >= lo) & (w < hi)
        if not sel.any():
            continue
        ts = t[sel].sum()
        out.append(f"| [{lo:.0e}, {hi:.0e}) | {sel.sum()} | {ts / 1e9:.2f} | {t[sel].mean() / 1e3:.1f} | "
                   f"{mx[sel].mean() / 1e3:.1f} | {w[sel].sum() / (ts / 1e3):.0f} | "
                   f"{tr['frontier'][sel].mean():.1f} |")
    return "\n".join(out)


def main(argv: list[str]) -> int:
    if len(argv) != 2:
        print(__doc__)
        return 2
    print(summary(load(argv[1])))
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
