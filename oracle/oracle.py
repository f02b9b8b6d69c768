"""ctypes bindings for the CPU oracle (``liboracle.so``) and for the
reference's own CPU code compiled here (``_ref/libref.so``).

TEST INFRASTRUCTURE ONLY: the test suite, the package smoke check and the CPU
baseline leg of the benchmark use this module to check or time the CUDA
engine.  The engine never imports it.

Graphs are passed as a dict of numpy arrays in the reference layout
(``src/graph/graph.h:43-51``): ``u_num``, ``l_num``, ``n``, ``m``,
``offsets`` (n+1), ``degrees`` (n), ``neighbors`` (2m), ``edges`` (2m),
``edge_ids`` (2m), all uint32.
"""

from __future__ import annotations

import ctypes as C
import os
import re
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libref.so")
# Root of the reference's source tree (read-only); only the recipes that
# compile or read the reference use it.
REF_ROOT = os.environ.get("BITRUSS_REFERENCE", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "src")

_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")


class _Graph(C.Structure):
    _fields_ = [
        ("n", C.c_uint32), ("u_num", C.c_uint32), ("m", C.c_uint64),
        ("offsets", C.c_void_p), ("neighbors", C.c_void_p), ("degrees", C.c_void_p),
        ("edges", C.c_void_p), ("edge_ids", C.c_void_p),
    ]


def build(ref: bool | None = None) -> None:
    """Compile liboracle.so (and _ref/libref.so when the reference sources
    are present, or when ``ref`` is True)."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    if ref or (ref is None and os.path.isdir(REF_SRC)):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_SRC}"], check=True)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(ref=False)
        L = C.CDLL(LIB_PATH)
        L.og_build_csr.restype = C.c_int
        L.og_build_csr.argtypes = [_u32p, _u32p, C.c_uint64, C.POINTER(C.c_uint32),
                                   C.POINTER(C.c_uint32), _u32p, _u32p, _u32p, _u32p, _u32p]
        L.og_ebfc.restype = None
        L.og_ebfc.argtypes = [C.POINTER(_Graph), C.c_int, _u64p, C.POINTER(C.c_uint64)]
        L.og_bfc.restype = C.c_uint64
        L.og_bfc.argtypes = [C.POINTER(_Graph), C.c_int]
        L.og_hidx.restype = C.c_uint32
        L.og_hidx.argtypes = [C.POINTER(_Graph), C.c_int, _u64p, _u64p]
        L.og_msp.restype = C.c_uint64
        L.og_msp.argtypes = [C.POINTER(_Graph), C.c_int, _u64p, C.c_int, _u64p, C.c_double]
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref():
    global _ref
    if _ref is None:
        L = C.CDLL(REF_PATH)
        L.ref_convert.restype = C.c_int
        L.ref_convert.argtypes = [C.c_char_p, C.c_char_p]
        L.ref_run.restype = C.c_longlong
        L.ref_run.argtypes = [C.c_char_p, C.c_int, C.c_int, _i64p, C.c_longlong, C.c_char_p]
        _ref = L
    return _ref


def build_csr(u: np.ndarray, v: np.ndarray) -> dict:
    """Reference CSR of an edge list in file order (graph.cpp:74-242)."""
    u = np.ascontiguousarray(u, dtype=np.uint32)
    v = np.ascontiguousarray(v, dtype=np.uint32)
    m = int(u.size)
    nmax = 2 * m + 1
    offsets = np.zeros(nmax + 1, np.uint32)
    degrees = np.zeros(nmax, np.uint32)
    nbr = np.zeros(max(2 * m, 1), np.uint32)
    edges = np.zeros(max(2 * m, 1), np.uint32)
    eids = np.zeros(max(2 * m, 1), np.uint32)
    un, ln = C.c_uint32(), C.c_uint32()
    rc = lib().og_build_csr(u, v, m, C.byref(un), C.byref(ln), offsets, degrees, nbr, edges, eids)
    if rc != 0:
        raise ValueError("vertex id >= MAX_IDS")
    n = un.value + ln.value
    return {
        "u_num": un.value, "l_num": ln.value, "n": n, "m": m,
        "offsets": offsets[: n + 1].copy(), "degrees": degrees[:n].copy(),
        "neighbors": nbr[: 2 * m].copy(), "edges": edges[: 2 * m].copy(),
        "edge_ids": eids[: 2 * m].copy(),
    }


def _gs(g: dict) -> _Graph:
    s = _Graph()
    s.n, s.u_num, s.m = g["n"], g["u_num"], g["m"]
    for k in ("offsets", "neighbors", "degrees", "edges", "edge_ids"):
        a = g[k]
        assert a.dtype == np.uint32 and a.flags.c_contiguous
        setattr(s, k, a.ctypes.data)
    return s


def ebfc(g: dict, threads: int = 0):
    """(uint64 supports[m], butterfly count) -- cpu_bfc.cpp:24-122."""
    sup = np.zeros(max(g["m"], 1), np.uint64)
    cnt = C.c_uint64()
    s = _gs(g)
    lib().og_ebfc(C.byref(s), threads, sup, C.byref(cnt))
    return sup[: g["m"]], cnt.value


def bfc(g: dict, threads: int = 0) -> int:
    s = _gs(g)
    return int(lib().og_bfc(C.byref(s), threads))


def hidx(g: dict, threads: int = 0, sup=None):
    """(uint64 bitruss[m], rounds) -- cpu_bitruss.cpp:152-266."""
    if sup is None:
        sup, _ = ebfc(g, threads)
    sup = np.ascontiguousarray(sup, dtype=np.uint64)
    if sup.size == 0:
        sup = np.zeros(1, np.uint64)
    out = np.zeros_like(sup)
    s = _gs(g)
    rounds = lib().og_hidx(C.byref(s), threads, sup, out)
    return out[: g["m"]], int(rounds)


MSP_REF, MSP_EXACT, MSP_TABLE, MSP_TABLE_EXACT = 0, 1, 2, 3


def msp(g: dict, threads: int = 0, mode: int = MSP_REF, sup=None, max_seconds: float = 0.0):
    """(uint64 bitruss[m], levels, stats) -- cpu_bitruss.cpp:563-624.

    stats = [levels, sub-rounds, compressions, peeled edges, row bytes,
    butterflies visited, unit decrements, algorithmic bytes]: the last four
    are the byte count of the reference's own peeling walk
    (bitruss_msp.cu:187-274; see og_msp in bt_oracle.c).  max_seconds > 0
    stops early (partial result, for bounded timing samples)."""
    if sup is None:
        sup, _ = ebfc(g, threads)
    work = np.array(sup, dtype=np.uint64, copy=True)
    if work.size == 0:
        work = np.zeros(1, np.uint64)
    stats = np.zeros(8, np.uint64)
    s = _gs(g)
    levels = lib().og_msp(C.byref(s), threads, work, mode, stats, max_seconds)
    return work[: g["m"]], int(levels), [int(x) for x in stats]


# --------------------------------------------------------------------------
# the reference's own CPU code (built here only)
# --------------------------------------------------------------------------

def ref_convert(text_path: str, bin_path: str) -> None:
    ref().ref_convert(text_path.encode(), bin_path.encode())


_ALGO = {"ebfc": 0, "bfc": 1, "hidx": 2, "msp": 3}


def ref_run(bin_path: str, algo: str, threads: int, m: int):
    """Run one reference CPU algorithm; returns (int64 result[m], log text)."""
    out = np.zeros(max(m, 1), np.int64)
    with tempfile.NamedTemporaryFile("r", suffix=".log") as lf:
        got = ref().ref_run(bin_path.encode(), _ALGO[algo], threads, out, out.size, lf.name.encode())
        if got < 0:
            raise RuntimeError("reference run failed")
        text = open(lf.name).read()
    return out[:m], text


def ref_log_count(text: str):
    """Butterfly count from a reference log ("butterfly count: N")."""
    mm = re.findall(r"butterfly count: ([\d,]+)", text)
    return int(mm[-1].replace(",", "")) if mm else None


def ref_log_levels(text: str):
    mm = re.findall(r"bitruss msp with ([\d,]+) levels", text)
    return int(mm[-1].replace(",", "")) if mm else None


def read_bin(path: str) -> dict:
    """Parse a reference .bin file (graph.cpp:293-375) with numpy."""
    raw = np.fromfile(path, dtype="<u4")
    u_num, l_num, u_max, m, smax = (int(x) for x in raw[:5])
    n = u_num + l_num
    pos = 5
    out = {"u_num": u_num, "l_num": l_num, "n": n, "m": m, "u_max": u_max, "support_max": smax}
    for k, ln in (("neighbors", 2 * m), ("offsets", n + 1), ("degrees", n),
                  ("edge_support", m), ("edges", 2 * m), ("edge_ids", 2 * m), ("bitruss", m)):
        out[k] = raw[pos: pos + ln].astype(np.uint32)
        pos += ln
    return out
