"""GB300 bitruss engine: Python mirror of the reference's host interface.

The engine is ``libbitruss.so`` (C ABI in ``include/bitruss.h``; CUDA kernels
for sm_103a).  This module binds it with ctypes and keeps the reference's
names (``src/graph/graph.h:30-52``, ``src/bfc/bfc.cuh:18-19``,
``src/bitruss/bitruss.cuh:17-18``):

    g = Graph.from_text("g.txt")          # Graph(path, true) / process_graph
    g.to_bin("g.bin")                      # graph_to_bin
    g = Graph.from_bin("g.bin")            # Graph(path, false) / load_graph_bin
    bfc_vpp(g)            -> g.butterflies
    bfc_evpp(g)           -> g.edge_support (uint64), g.support_max
    g_bitruss_hindex(g)   -> g.bitruss (uint32), g.rounds
    bitruss_msp(g)        -> g.bitruss (uint32), g.levels

Failures raise ``BitrussError`` (the reference calls exit()).  There is no CPU
fallback: without the built library or a GB300 the calls raise.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

__all__ = [
    "BitrussError", "Graph", "Context", "load", "build",
    "bfc_vpp", "bfc_evpp", "g_bitruss_hindex", "bitruss_msp", "bitruss_msp_exact", "bfc_noalloc",
    "pack", "Server", "OPS",
    "STATUS", "SYMBOLS",
]

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libbitruss.so")
COH_PATH = os.path.join(PKG, "coh")

STATUS = {
    0: "BT_OK", 1: "BT_ERR_INVALID", 2: "BT_ERR_IO", 3: "BT_ERR_FORMAT",
    4: "BT_ERR_HOST_MEMORY", 5: "BT_ERR_DEVICE_MEMORY", 6: "BT_ERR_CUDA",
    7: "BT_ERR_TIMEOUT", 8: "BT_ERR_STATE", 9: "BT_ERR_NO_DEVICE", 10: "BT_ERR_OVERFLOW",
}

# every symbol include/bitruss.h declares
SYMBOLS = [
    "bt_graph_load_bin", "bt_graph_load_text", "bt_graph_from_edges", "bt_graph_save_bin",
    "bt_graph_get_view", "bt_graph_free", "bt_ctx_create", "bt_ctx_set_stream",
    "bt_ctx_set_memory_budget", "bt_ctx_memory_used", "bt_ctx_free", "bt_graph_upload",
    "bt_bfc", "bt_ebfc", "bt_hidx", "bt_msp", "bt_msp_exact", "bt_result_download",
    "bt_ctx_phase_ms", "bt_ctx_stats", "bt_status_string", "bt_last_error",
    "bt_bfc_noalloc",
    "bt_ctx_set_msp_schedule", "bt_ctx_get_msp_schedule", "bt_msp_autotune",
    "bt_graph_pack", "bt_ctx_set_arena_edges", "bt_ctx_set_peel_ctas", "bt_msp_batch", "bt_ebfc_batch",
    "bt_ctx_memory_peak", "bt_server_create", "bt_server_submit", "bt_server_wait",
    "bt_server_latency", "bt_server_stats", "bt_server_free", "bt_job_bytes",
    "bt_kernel_launches",
]

OPS = {"bfc": 0, "ebfc": 1, "msp": 2, "msp_exact": 3}


class BitrussError(RuntimeError):
    def __init__(self, status: int, where: str, message: str):
        self.status = status
        self.code = STATUS.get(status, str(status))
        super().__init__(f"{where}: {self.code}: {message}")


class _View(C.Structure):
    _fields_ = [
        ("u_num", C.c_uint32), ("l_num", C.c_uint32), ("u_max", C.c_uint32), ("n", C.c_uint32),
        ("m", C.c_uint64), ("support_max", C.c_uint64),
        ("offsets", C.c_void_p), ("neighbors", C.c_void_p), ("degrees", C.c_void_p),
        ("edges", C.c_void_p), ("edge_ids", C.c_void_p),
    ]


class _RequestInfo(C.Structure):
    _fields_ = [
        ("status", C.c_int), ("count", C.c_uint64), ("support_max", C.c_uint64),
        ("levels", C.c_uint32), ("batch_size", C.c_uint32),
        ("queue_ms", C.c_double), ("run_ms", C.c_double), ("total_ms", C.c_double),
    ]


_lib = None


def build(verbose: bool = False) -> str:
    from . import _build
    return _build.build(verbose=verbose)


def load():
    """Load libbitruss.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise BitrussError(9, "load", f"{LIB_PATH} is missing: build it with "
                           "gpu_bitruss_gb300.build() (nvcc for sm_103a)")
    L = C.CDLL(LIB_PATH)
    P, u32, u64, i32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int
    sig = {
        "bt_graph_load_bin": ([C.c_char_p, C.POINTER(P)], i32),
        "bt_graph_load_text": ([C.c_char_p, C.POINTER(P)], i32),
        "bt_graph_from_edges": ([P, P, u64, C.POINTER(P)], i32),
        "bt_graph_save_bin": ([P, C.c_char_p], i32),
        "bt_graph_get_view": ([P, C.POINTER(_View)], i32),
        "bt_graph_free": ([P], None),
        "bt_ctx_create": ([i32, C.POINTER(P)], i32),
        "bt_ctx_set_stream": ([P, P], i32),
        "bt_ctx_set_memory_budget": ([P, u64], i32),
        "bt_ctx_memory_used": ([P, C.POINTER(u64)], i32),
        "bt_ctx_free": ([P], None),
        "bt_graph_upload": ([P, P], i32),
        "bt_bfc": ([P, C.POINTER(u64)], i32),
        "bt_ebfc": ([P, P, C.POINTER(u64), C.POINTER(u64)], i32),
        "bt_hidx": ([P, P, C.POINTER(u32)], i32),
        "bt_msp": ([P, P, C.POINTER(u32)], i32),
        "bt_msp_exact": ([P, P, C.POINTER(u32)], i32),
        "bt_result_download": ([P, P, C.c_size_t], i32),
        "bt_ctx_phase_ms": ([P, C.c_char_p], C.c_double),
        "bt_ctx_stats": ([P, C.POINTER(u64), i32], i32),
        "bt_status_string": ([i32], C.c_char_p),
        "bt_last_error": ([], C.c_char_p),
        "bt_bfc_noalloc": ([i32, P, P, u32, u64, P, P], i32),
        "bt_ctx_set_msp_schedule": ([P, u32, u32, u32], i32),
        "bt_ctx_get_msp_schedule": ([P, P], i32),
        "bt_msp_autotune": ([P, P, C.POINTER(C.c_double)], i32),
        "bt_graph_pack": ([P, u32, C.POINTER(P), P], i32),
        "bt_ctx_set_arena_edges": ([P, u64], i32),
        "bt_ctx_set_peel_ctas": ([P, u32], i32),
        "bt_msp_batch": ([P, P, u32, i32, P, P], i32),
        "bt_ebfc_batch": ([P, P, u32, P, P], i32),
        "bt_ctx_memory_peak": ([P, C.POINTER(u64), i32], i32),
        "bt_server_create": ([i32, u32, u64, C.POINTER(P)], i32),
        "bt_server_submit": ([P, P, i32, P, C.POINTER(u64)], i32),
        "bt_server_wait": ([P, u64, C.c_double, C.POINTER(_RequestInfo)], i32),
        "bt_server_latency": ([P, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(u64), i32], i32),
        "bt_server_stats": ([P, C.POINTER(u64), i32], i32),
        "bt_server_free": ([P], None),
        "bt_job_bytes": ([P, P, u32, i32, C.POINTER(u64)], i32),
        "bt_kernel_launches": ([], u64),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def _check(rc: int, where: str) -> None:
    if rc != 0:
        msg = load().bt_last_error().decode(errors="replace")
        raise BitrussError(rc, where, msg)


def _ptr(a: np.ndarray | None):
    return None if a is None else C.c_void_p(a.ctypes.data)


class Graph:
    """Host CSR in the reference layout (graph.h:43-51)."""

    def __init__(self, handle):
        self._h = handle
        self.edge_support = None   # np.uint64[m] after bfc_evpp
        self.bitruss = None        # np.uint32[m] after hidx / msp
        self.butterflies = None
        self.levels = None
        self.rounds = None
        self._refresh()

    # constructors -------------------------------------------------------
    @classmethod
    def from_edges(cls, u, v) -> "Graph":
        u = np.ascontiguousarray(u, dtype=np.uint32)
        v = np.ascontiguousarray(v, dtype=np.uint32)
        if u.shape != v.shape:
            raise ValueError("u and v differ in length")
        h = C.c_void_p()
        _check(load().bt_graph_from_edges(_ptr(u), _ptr(v), u.size, C.byref(h)), "process_graph")
        return cls(h)

    @classmethod
    def from_text(cls, path: str) -> "Graph":
        h = C.c_void_p()
        _check(load().bt_graph_load_text(path.encode(), C.byref(h)), "process_graph")
        return cls(h)

    @classmethod
    def from_bin(cls, path: str) -> "Graph":
        h = C.c_void_p()
        _check(load().bt_graph_load_bin(path.encode(), C.byref(h)), "load_graph_bin")
        return cls(h)

    def to_bin(self, path: str) -> None:
        _check(load().bt_graph_save_bin(self._h, path.encode()), "graph_to_bin")

    graph_to_bin = to_bin

    def _refresh(self):
        v = _View()
        _check(load().bt_graph_get_view(self._h, C.byref(v)), "graph view")
        self.u_num, self.l_num, self.u_max, self.n, self.m = v.u_num, v.l_num, v.u_max, v.n, v.m
        self.support_max = v.support_max

        def arr(p, k):
            if k == 0 or not p:
                return np.zeros(0, np.uint32)
            return np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_uint32)), shape=(k,))

        self.offsets = arr(v.offsets, self.n + 1)
        self.neighbors = arr(v.neighbors, 2 * self.m)
        self.degrees = arr(v.degrees, self.n)
        self.edges = arr(v.edges, 2 * self.m)
        self.edge_ids = arr(v.edge_ids, 2 * self.m)

    def as_dict(self) -> dict:
        """Arrays as a dict (the layout the CPU oracle takes)."""
        return {"u_num": self.u_num, "l_num": self.l_num, "n": self.n, "m": self.m,
                "offsets": self.offsets, "degrees": self.degrees, "neighbors": self.neighbors,
                "edges": self.edges, "edge_ids": self.edge_ids}

    def close(self):
        if getattr(self, "_h", None):
            load().bt_graph_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Context:
    """A device context: one stream, one resident graph."""

    def __init__(self, device: int = 0):
        self._c = C.c_void_p()
        _check(load().bt_ctx_create(device, C.byref(self._c)), "bt_ctx_create")
        self.graph = None

    def set_stream(self, stream_ptr: int | None) -> None:
        _check(load().bt_ctx_set_stream(self._c, C.c_void_p(stream_ptr or 0)), "set_stream")

    def set_budget(self, nbytes: int) -> None:
        _check(load().bt_ctx_set_memory_budget(self._c, nbytes), "set_budget")

    def memory_used(self) -> int:
        x = C.c_uint64()
        _check(load().bt_ctx_memory_used(self._c, C.byref(x)), "memory_used")
        return x.value

    def memory_peak(self, reset: bool = False) -> int:
        x = C.c_uint64()
        _check(load().bt_ctx_memory_peak(self._c, C.byref(x), 1 if reset else 0), "memory_peak")
        return x.value

    def job_bytes(self, graphs: list, op: str) -> int:
        """The server's admission estimate for one arena of `graphs` and `op`."""
        hs, _ = _handles(graphs)
        x = C.c_uint64()
        _check(load().bt_job_bytes(self._c, hs, len(graphs), OPS[op], C.byref(x)), "job_bytes")
        return x.value

    def upload(self, g: Graph) -> None:
        _check(load().bt_graph_upload(self._c, g._h), "graph upload")
        self.graph = g

    def bfc(self) -> int:
        c = C.c_uint64()
        _check(load().bt_bfc(self._c, C.byref(c)), "bfc_vpp")
        return c.value

    def ebfc(self, out: bool = True):
        m = self.graph.m
        sup = np.zeros(m, np.uint64) if out else None
        c, mx = C.c_uint64(), C.c_uint64()
        _check(load().bt_ebfc(self._c, _ptr(sup) if m else None, C.byref(c), C.byref(mx)), "bfc_evpp")
        return sup, c.value, mx.value

    def hidx(self, out: bool = True):
        m = self.graph.m
        b = np.zeros(m, np.uint32) if out else None
        r = C.c_uint32()
        _check(load().bt_hidx(self._c, _ptr(b) if m else None, C.byref(r)), "g_bitruss_hindex")
        return b, r.value

    def msp(self, exact: bool = False, out: bool = True, into: np.ndarray | None = None):
        """Bitruss numbers of the resident graph (into `into` when given,
        a uint32 array of at least m entries) and the level count."""
        m = self.graph.m
        if into is not None:
            if into.dtype != np.uint32 or into.size < m or not into.flags.c_contiguous:
                raise ValueError("into must be a contiguous uint32 array of at least m entries")
            b = into
        else:
            b = np.zeros(m, np.uint32) if out else None
        lv = C.c_uint32()
        f = load().bt_msp_exact if exact else load().bt_msp
        _check(f(self._c, _ptr(b) if m else None, C.byref(lv)), "bitruss_msp")
        return b, lv.value

    # schedule and autotuner ------------------------------------------------
    def set_msp_schedule(self, min_grain: int = 0, tasks_per_cta: int = 0, local_plan: int = 0) -> None:
        _check(load().bt_ctx_set_msp_schedule(self._c, min_grain, tasks_per_cta, local_plan),
               "set_msp_schedule")

    def msp_schedule(self) -> tuple[int, int, int]:
        a = np.zeros(3, np.uint32)
        _check(load().bt_ctx_get_msp_schedule(self._c, _ptr(a)), "msp_schedule")
        return tuple(int(x) for x in a)

    def autotune(self) -> tuple[tuple[int, int, int], float]:
        """Tune the msp schedule on the resident graph; returns (schedule, kernel ms)."""
        a = np.zeros(3, np.uint32)
        ms = C.c_double()
        _check(load().bt_msp_autotune(self._c, _ptr(a), C.byref(ms)), "msp autotune")
        return tuple(int(x) for x in a), ms.value

    def set_peel_ctas(self, ctas: int) -> None:
        """CTAs of the peeling kernel (0: one per SM, the whole GPU)."""
        _check(load().bt_ctx_set_peel_ctas(self._c, ctas), "set_peel_ctas")

    # batched arenas ----------------------------------------------------------
    def set_arena_edges(self, edges: int) -> None:
        _check(load().bt_ctx_set_arena_edges(self._c, edges), "set_arena_edges")

    def msp_batch(self, graphs: list, exact: bool = False):
        """Bitruss numbers of every graph (one array each) and their level counts."""
        hs, base = _handles(graphs)
        b = np.zeros(max(int(base[-1]), 1), np.uint32)
        lv = np.zeros(max(len(graphs), 1), np.uint32)
        _check(load().bt_msp_batch(self._c, hs, len(graphs), 1 if exact else 0, _ptr(b), _ptr(lv)),
               "msp batch")
        self.graph = None  # the context now holds the last arena
        return [b[base[i]:base[i + 1]] for i in range(len(graphs))], lv[:len(graphs)]

    def ebfc_batch(self, graphs: list):
        """Supports of every graph (one array each) and their butterfly counts."""
        hs, base = _handles(graphs)
        sup = np.zeros(max(int(base[-1]), 1), np.uint64)
        cnt = np.zeros(max(len(graphs), 1), np.uint64)
        _check(load().bt_ebfc_batch(self._c, hs, len(graphs), _ptr(sup), _ptr(cnt)), "ebfc batch")
        self.graph = None
        return [sup[base[i]:base[i + 1]] for i in range(len(graphs))], cnt[:len(graphs)]

    def download(self, out: np.ndarray) -> None:
        _check(load().bt_result_download(self._c, _ptr(out), out.nbytes), "result download")

    def phase_ms(self, phase: str) -> float:
        return float(load().bt_ctx_phase_ms(self._c, phase.encode()))

    def stats(self) -> list[int]:
        """[levels, sub-rounds, compressions, tasks, hidx rounds, non-empty
        levels, bucket splits, -, peel tasks run, probes, anchor slots,
        butterflies found, decrements, m, ns in level transitions, ns in
        peel phases, ns in finalize phases, bytes per working support (4 or 8),
        -, -, then SM cycles per CTA
        of the peeling kernel by step: task, stage, slice, probe, hits, flush,
        barrier, other]"""
        a = (C.c_uint64 * 28)()
        _check(load().bt_ctx_stats(self._c, a, 28), "stats")
        return list(a)

    def close(self):
        if getattr(self, "_c", None):
            load().bt_ctx_free(self._c)
            self._c = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Request loop (bt_server_*): submit graphs with an op, wait for tickets."""

    def __init__(self, device: int = 0, slots: int = 2, hbm_budget: int = 0):
        self._s = C.c_void_p()
        _check(load().bt_server_create(device, slots, hbm_budget, C.byref(self._s)), "bt_server_create")
        self._keep = {}

    def submit(self, g: Graph, op: str):
        """Queue a request; returns (ticket, output array or None)."""
        out = None
        if op in ("msp", "msp_exact"):
            out = np.zeros(max(g.m, 1), np.uint32)
        elif op == "ebfc":
            out = np.zeros(max(g.m, 1), np.uint64)
        t = C.c_uint64()
        _check(load().bt_server_submit(self._s, g._h, OPS[op], _ptr(out), C.byref(t)), "server submit")
        self._keep[t.value] = (g, out)
        return t.value, (out[:g.m] if out is not None else None)

    def wait(self, ticket: int, timeout_ms: float = -1.0) -> dict:
        info = _RequestInfo()
        rc = load().bt_server_wait(self._s, ticket, timeout_ms, C.byref(info))
        if rc != 7:  # BT_ERR_TIMEOUT keeps the ticket
            self._keep.pop(ticket, None)
        _check(rc, "server wait")
        return {k: getattr(info, k) for k, _ in _RequestInfo._fields_}

    def latency(self, reset: bool = False) -> tuple[float, float, int]:
        p50, p99, n = C.c_double(), C.c_double(), C.c_uint64()
        _check(load().bt_server_latency(self._s, C.byref(p50), C.byref(p99), C.byref(n), 1 if reset else 0),
               "server latency")
        return p50.value, p99.value, n.value

    def stats(self) -> dict:
        a = (C.c_uint64 * 6)()
        _check(load().bt_server_stats(self._s, a, 6), "server stats")
        return dict(zip(["budget", "reserved", "running", "queued", "batches", "batched_requests"], list(a)))

    def close(self):
        if getattr(self, "_s", None):
            load().bt_server_free(self._s)
            self._s = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _handles(graphs: list):
    arr = (C.c_void_p * max(len(graphs), 1))(*[g._h for g in graphs])
    base = np.zeros(len(graphs) + 1, np.int64)
    base[1:] = np.cumsum([g.m for g in graphs]) if graphs else []
    return arr, base


def pack(graphs: list) -> tuple["Graph", np.ndarray]:
    """The arena of a batched call as a host graph, with each graph's first edge id."""
    hs, _ = _handles(graphs)
    base = np.zeros(len(graphs) + 1, np.uint64)
    h = C.c_void_p()
    _check(load().bt_graph_pack(hs, len(graphs), C.byref(h), _ptr(base)), "graph pack")
    return Graph(h), base


_default_ctx: Context | None = None


def _ctx_for(g: Graph) -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    if _default_ctx.graph is not g:
        _default_ctx.upload(g)
    return _default_ctx


def bfc_vpp(g: Graph) -> int:
    """Global butterfly count (bfc_vpp.cu:321-385)."""
    g.butterflies = _ctx_for(g).bfc()
    return g.butterflies


def bfc_evpp(g: Graph) -> np.ndarray:
    """Per-edge butterfly support (bfc_vpp.cu:233-309)."""
    sup, c, mx = _ctx_for(g).ebfc()
    g.edge_support, g.butterflies, g.support_max = sup, c, mx
    return sup


def g_bitruss_hindex(g: Graph) -> np.ndarray:
    """Bitruss numbers by h-index iteration (bitruss_hidx.cu:179-256)."""
    b, r = _ctx_for(g).hidx()
    g.bitruss, g.rounds = b, r
    return b


def bitruss_msp(g: Graph) -> np.ndarray:
    """Bitruss numbers by multi-stage peeling (bitruss_msp.cu:440-583)."""
    b, lv = _ctx_for(g).msp()
    g.bitruss, g.levels = b, lv
    return b


def bfc_noalloc(device: int, d_offsets: int, d_neighbors: int, n: int, m: int,
                d_count: int, stream: int = 0) -> None:
    """Butterfly count into caller-owned device buffers (raw device pointers),
    without any device allocation by the library; enqueued on `stream`."""
    _check(load().bt_bfc_noalloc(device, C.c_void_p(d_offsets), C.c_void_p(d_neighbors), n, m,
                                 C.c_void_p(d_count), C.c_void_p(stream or 0)), "bt_bfc_noalloc")


def kernel_launches() -> int:
    """The library's own kernel launches in this process so far."""
    return int(load().bt_kernel_launches())


def bitruss_msp_exact(g: Graph) -> np.ndarray:
    """Peeling with the corrected one-survivor rule (equals hidx)."""
    b, lv = _ctx_for(g).msp(exact=True)
    g.bitruss, g.levels = b, lv
    return b
