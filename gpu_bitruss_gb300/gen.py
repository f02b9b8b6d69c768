"""Seeded synthetic bipartite graphs for the bitruss workloads.

The reference ships no generator and no benchmark graphs (its only data file is
``data/aw.graph``), so every workload here is synthetic.  Each generator returns
the edge list in *draw order* as two ``uint32`` arrays ``(u, v)``: ``u`` is a
U-side (upper) id and ``v`` a V-side (lower) id, exactly the two columns of the
reference's ``u v`` text format (``src/graph/graph.cpp:92-114``).  The order
matters: the reference numbers vertices by first appearance and edges by rank
in U-major sorted order (``graph.cpp:99-105``, ``:178-194``), and the msp tie
rule depends on edge ids, so the same arrays must feed both the engine and the
oracle.

Randomness is numpy ``Generator(PCG64(seed))``.  Duplicate pairs are rejected:
the first occurrence of each (u, v) pair is kept, in draw order, until ``m``
unique edges exist.

Workloads (sizes are the defaults of each function):

* ``er``        uniform bipartite, |U|=2,000, |V|=3,000, m=20,000, seed 1.
* ``chung_lu``  power-law bipartite: vertex i of a side has weight
                proportional to (i+1)^(-1/(gamma-1)); the weights are scaled to
                sum to m and capped (cap, rescale, repeat until no weight is
                above the cap); endpoints are drawn by inverse-CDF sampling
                (``searchsorted`` on the cumulative weights).
                Config "cl20m": |U|=1,000,000, |V|=500,000, m=20,000,000,
                gamma=2.1 on both sides, cap 50,000, seed 2.
* ``hub_skew``  U side power law (gamma=1.8, cap 1,000,000, |U|=100,000),
                V side uniform (|V|=5,000,000), m=100,000,000, seed 3.
* ``batch``     the i-th graph of the 4,096-graph batch: m_i log-uniform in
                [1e3, 2e6], |U|:|V| ratio uniform in [0.2, 5], |U|+|V| chosen
                so the mean degree is 8 (min 8 vertices per side), Chung-Lu
                gamma=2.3, seed 4+i.
"""

from __future__ import annotations

import hashlib

import numpy as np

__all__ = [
    "er",
    "chung_lu",
    "hub_skew",
    "batch_graph",
    "batch_sizes",
    "power_weights",
    "by_name",
    "digest",
    "to_text",
]


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def _unique_in_order(keys: np.ndarray) -> np.ndarray:
    """Unique values of ``keys`` in order of first occurrence."""
    _, first = np.unique(keys, return_index=True)
    first.sort()
    return keys[first]


def _draw_unique(draw, m: int, nv: int) -> tuple[np.ndarray, np.ndarray]:
    """Draw (u, v) batches with ``draw(count)`` until ``m`` unique pairs exist.

    Pairs are packed as ``u * nv + v`` (int64).  The first occurrence of each
    pair is kept, in draw order.
    """
    accepted = np.empty(0, dtype=np.int64)
    accepted_sorted = np.empty(0, dtype=np.int64)
    need = m
    while need > 0:
        batch = max(int(need * 1.25) + 1024, 4096)
        u, v = draw(batch)
        keys = _unique_in_order(u.astype(np.int64) * nv + v.astype(np.int64))
        if accepted_sorted.size:
            pos = np.searchsorted(accepted_sorted, keys)
            pos[pos == accepted_sorted.size] = 0
            keys = keys[accepted_sorted[pos] != keys]
        keys = keys[:need]
        accepted = np.concatenate([accepted, keys])
        accepted_sorted = np.sort(accepted)
        need = m - accepted.size
    u = (accepted // nv).astype(np.uint32)
    v = (accepted % nv).astype(np.uint32)
    return u, v


def er(nu: int = 2000, nv: int = 3000, m: int = 20000, seed: int = 1):
    """Erdos-Renyi bipartite graph with ``m`` unique edges drawn uniformly."""
    if m > nu * nv:
        raise ValueError("more edges than vertex pairs")
    rng = _rng(seed)

    def draw(k):
        return rng.integers(0, nu, size=k), rng.integers(0, nv, size=k)

    return _draw_unique(draw, m, nv)


def power_weights(n: int, gamma: float, total: float, cap: float) -> np.ndarray:
    """Chung-Lu expected degrees: (i+1)^(-1/(gamma-1)) scaled to ``total``.

    Weights above ``cap`` are clamped to it and the uncapped ones rescaled so
    the sum stays ``total``; this repeats until no weight exceeds the cap.
    """
    w = np.arange(1, n + 1, dtype=np.float64) ** (-1.0 / (gamma - 1.0))
    w *= total / w.sum()
    for _ in range(200):
        over = w > cap
        if not over.any():
            break
        w[over] = cap
        free = ~over & (w < cap)
        rest = total - cap * np.count_nonzero(w >= cap)
        if rest <= 0 or not free.any():
            break
        w[free] *= rest / w[free].sum()
    return w


def _cdf(w: np.ndarray) -> np.ndarray:
    c = np.cumsum(w)
    return c / c[-1]


def chung_lu(nu: int = 1_000_000, nv: int = 500_000, m: int = 20_000_000,
             gamma_u: float = 2.1, gamma_v: float = 2.1,
             cap_u: float = 50_000, cap_v: float = 50_000, seed: int = 2):
    """Chung-Lu power-law bipartite graph with ``m`` unique edges."""
    cu = _cdf(power_weights(nu, gamma_u, m, cap_u))
    cv = _cdf(power_weights(nv, gamma_v, m, cap_v))
    rng = _rng(seed)

    def draw(k):
        u = np.searchsorted(cu, rng.random(k), side="right")
        v = np.searchsorted(cv, rng.random(k), side="right")
        np.minimum(u, nu - 1, out=u)
        np.minimum(v, nv - 1, out=v)
        return u, v

    return _draw_unique(draw, m, nv)


def hub_skew(nu: int = 100_000, nv: int = 5_000_000, m: int = 100_000_000,
             gamma_u: float = 1.8, cap_u: float = 1_000_000, seed: int = 3):
    """Hub-skewed graph: power-law U side, uniform V side."""
    cu = _cdf(power_weights(nu, gamma_u, m, cap_u))
    rng = _rng(seed)

    def draw(k):
        u = np.searchsorted(cu, rng.random(k), side="right")
        np.minimum(u, nu - 1, out=u)
        return u, rng.integers(0, nv, size=k)

    return _draw_unique(draw, m, nv)


def batch_sizes(count: int = 4096, lo: float = 1e3, hi: float = 2e6, seed: int = 4):
    """Per-graph (m, |U|, |V|) of the batched workload (log-uniform m)."""
    rng = _rng(seed)
    m = np.exp(rng.uniform(np.log(lo), np.log(hi), size=count)).astype(np.int64)
    ratio = rng.uniform(0.2, 5.0, size=count)
    verts = np.maximum(m // 4, 16)          # mean degree 8 over |U|+|V|
    nu = np.maximum((verts * ratio / (1.0 + ratio)).astype(np.int64), 8)
    nv = np.maximum(verts - nu, 8)
    return m, nu, nv


def batch_graph(i: int, count: int = 4096, sizes=None):
    """The i-th graph of the batched workload (Chung-Lu, gamma 2.3, seed 4+i)."""
    m, nu, nv = sizes if sizes is not None else batch_sizes(count)
    mi, nui, nvi = int(m[i]), int(nu[i]), int(nv[i])
    cap = max(8.0, float(min(nui, nvi)) * 0.5)
    return chung_lu(nui, nvi, mi, 2.3, 2.3, min(cap, nvi), min(cap, nui), seed=4 + i)


def by_name(name: str):
    """Named workloads: aw (the reference's fixture), er, cl20m, hub100m,
    scaled-down Chung-Lu cases cl<k>k and scaled-down hub-skewed cases
    hub<k>k (k thousand edges) for tests."""
    if name == "er":
        return er()
    if name == "cl20m":
        return chung_lu()
    if name == "hub100m":
        return hub_skew()
    if name.startswith("hub") and name.endswith("k") and name[3:-1].isdigit():
        # the hub100m shape scaled to k thousand edges: |U|, |V| and the hub
        # cap scale with m, the mean V degree (20) stays
        k = int(name[3:-1]) * 1000
        scale = k / 100_000_000
        return hub_skew(max(int(100_000 * scale), 16), max(int(5_000_000 * scale), 16), k,
                        1.8, max(1_000_000 * scale, 16.0), seed=3)
    if name.startswith("cl") and name.endswith("k") and name[2:-1].isdigit():
        k = int(name[2:-1]) * 1000
        # same shape as cl20m, vertex counts scaled with m
        scale = k / 20_000_000
        nu = max(int(1_000_000 * scale), 64)
        nv = max(int(500_000 * scale), 32)
        cap = max(50_000 * scale ** 0.5, 16)
        return chung_lu(nu, nv, k, 2.1, 2.1, min(cap, nv), min(cap, nu), seed=2)
    raise KeyError(name)


def digest(u: np.ndarray, v: np.ndarray) -> str:
    """Order-sensitive digest of an edge list (sha256 of the u32 columns)."""
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(u, dtype="<u4").tobytes())
    h.update(np.ascontiguousarray(v, dtype="<u4").tobytes())
    return h.hexdigest()[:16]


def to_text(path: str, u: np.ndarray, v: np.ndarray) -> None:
    """Write ``u v`` lines (the reference's input text format)."""
    with open(path, "w") as f:
        for a, b in zip(u.tolist(), v.tolist()):
            f.write(f"{a} {b}\n")
