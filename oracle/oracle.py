"""ORACLE -- test infrastructure only.

CPU checker of the segmented sort.  Imported only by tests/, by
__graft_entry__.smoke() and by bench.py's CPU-baseline leg; the GPU library
never imports or calls it, and nothing here is a fallback for it.

Two restatements of the reference's per-segment stable sort
(src/mseq.cu:44-49 `segmented_sorting`; src/bb_segsort/main.cu:152-173
`gold_segsort`, a stable sort of (key, value) pairs comparing keys only):

* ``segsort_cpp``  -- ctypes binding of segsort_oracle.cpp (std::stable_sort
  per segment, optionally over several std::threads);
* ``segsort_numpy`` -- one numpy ``lexsort`` over (order bits, segment id),
  which is stable, so it gives the same order; fast enough for 2^24-element
  checks.

Both compare keys through the library's order-preserving bits (``order_bits``)
and follow its offsets contract (CSR, every offset clamped into [0, n], a
segment whose end is below its begin is empty).  The restatement is pinned
against the reference's own ``mseq`` program (built from its sources by
``make -C oracle ref``) and against the committed fixtures in tests/golden/.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"
REF_MSEQ = HERE / "_ref" / "mseq.exe"
REF_FIXSEQ = HERE / "_ref" / "fixseq.exe"

_KEY_SUFFIX = {np.dtype(np.uint32): "u32", np.dtype(np.int32): "i32",
               np.dtype(np.float32): "f32", np.dtype(np.uint64): "u64"}
_CTYPE = {"u32": ctypes.c_uint32, "i32": ctypes.c_int32,
          "f32": ctypes.c_float, "u64": ctypes.c_uint64}

_lib = None


def build() -> None:
    """Compile liboracle.so (g++) with the recipe in oracle/Makefile."""
    import subprocess
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = ctypes.CDLL(str(LIB_PATH))
        for suf, ct in _CTYPE.items():
            P = ctypes.POINTER(ct)
            fk = getattr(L, f"oracle_segsort_keys_{suf}")
            fk.argtypes = [P, ctypes.c_int64, ctypes.POINTER(ctypes.c_int32),
                           ctypes.c_int32, ctypes.c_int]
            fk.restype = None
            fp = getattr(L, f"oracle_segsort_pairs_{suf}")
            fp.argtypes = [P, ctypes.POINTER(ctypes.c_uint32), ctypes.c_int64,
                           ctypes.POINTER(ctypes.c_int32), ctypes.c_int32, ctypes.c_int]
            fp.restype = None
        _lib = L
    return _lib


def order_bits(keys: np.ndarray) -> np.ndarray:
    """Order-preserving unsigned bits of the keys (the library's key order)."""
    dt = keys.dtype
    if dt == np.uint32 or dt == np.uint64:
        return keys
    if dt == np.int32:
        return keys.view(np.uint32) ^ np.uint32(0x80000000)
    if dt == np.float32:
        u = keys.view(np.uint32)
        neg = (u & np.uint32(0x80000000)) != 0
        return np.where(neg, ~u, u ^ np.uint32(0x80000000)).astype(np.uint32)
    raise TypeError(f"unsupported key dtype {dt}")


def heads_to_csr(heads: np.ndarray, n: int) -> np.ndarray:
    """Heads-only offsets (last segment ends at n) -> CSR offsets."""
    return np.concatenate([np.asarray(heads, dtype=np.int32), np.array([n], np.int32)])


def segsort_cpp(keys: np.ndarray, offsets: np.ndarray, vals: np.ndarray | None = None,
                threads: int = 1):
    """Per-segment std::stable_sort (segsort_oracle.cpp).  Returns new arrays."""
    suf = _KEY_SUFFIX[keys.dtype]
    k = np.ascontiguousarray(keys).copy()
    o = np.ascontiguousarray(offsets, dtype=np.int32)
    nseg = len(o) - 1
    P = ctypes.POINTER(_CTYPE[suf])
    kp = k.ctypes.data_as(P)
    op = o.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
    if vals is None:
        getattr(lib(), f"oracle_segsort_keys_{suf}")(kp, len(k), op, nseg, threads)
        return k
    v = np.ascontiguousarray(vals, dtype=np.uint32).copy()
    getattr(lib(), f"oracle_segsort_pairs_{suf}")(
        kp, v.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), len(k), op, nseg, threads)
    return k, v


def segsort_numpy(keys: np.ndarray, offsets: np.ndarray, vals: np.ndarray | None = None,
                  descending: bool = False):
    """Same result as segsort_cpp via one stable lexsort.  Returns new arrays.

    descending=True sorts every segment by decreasing key, equal keys in input
    order (the stable descending order of CUB's SortPairsDescending,
    lib/cub/device/device_segmented_radix_sort.cuh:338).  Values keep their
    dtype (32- or 64-bit)."""
    n = len(keys)
    o = np.clip(np.asarray(offsets, dtype=np.int64), 0, n)
    b, e = o[:-1], o[1:]
    lens = np.maximum(e - b, 0)
    k = np.array(keys, copy=True)
    if vals is not None and np.asarray(vals).dtype not in (np.dtype(np.uint32), np.dtype(np.uint64)):
        vals = np.asarray(vals, dtype=np.uint32)
    v = None if vals is None else np.array(vals, copy=True)
    if n == 0 or lens.sum() == 0:
        return k if v is None else (k, v)
    # Positions covered by a segment, in segment order, and their segment ids.
    seg_ids = np.repeat(np.arange(len(lens), dtype=np.int64), lens)
    starts = np.repeat(b, lens)
    within = np.arange(len(seg_ids), dtype=np.int64) - np.repeat(np.cumsum(lens) - lens, lens)
    pos = starts + within
    bits = order_bits(keys[pos])
    if descending:
        bits = ~bits
    order = np.lexsort((bits, seg_ids))  # stable: ties keep position order
    k[pos] = keys[pos][order]
    if v is not None:
        v[pos] = np.asarray(vals)[pos][order]
        return k, v
    return k


def c1_text(offsets: np.ndarray, keys: np.ndarray) -> str:
    """Instance in the reference's text format (utils/gen_equal.cpp:108-114):
    nseg, the nseg+1 offsets, n, the n keys."""
    nseg = len(offsets) - 1
    return (f"{nseg}\n" + " ".join(str(int(x)) for x in offsets) + " \n"
            + f"{len(keys)}\n" + " ".join(str(int(x)) for x in keys) + " \n")


def run_reference_mseq(offsets: np.ndarray, keys: np.ndarray) -> np.ndarray:
    """Run the reference's own mseq program (built by `make -C oracle ref`)
    on one instance and parse the sorted keys it prints (src/mseq.cu:27-33)."""
    import subprocess
    if not REF_MSEQ.exists():
        raise FileNotFoundError(f"{REF_MSEQ} not built (make -C oracle ref)")
    out = subprocess.run([str(REF_MSEQ)], input=c1_text(offsets, keys), text=True,
                         capture_output=True, check=True).stdout
    return np.array(out.split(), dtype=np.int64).astype(np.uint32)


def default_threads() -> int:
    return max(1, len(os.sched_getaffinity(0)))
