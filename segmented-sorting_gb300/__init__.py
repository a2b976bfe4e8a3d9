"""GB300 segmented sort -- Python host side.

A thin ctypes layer over the C ABI in include/segsort.h (libsegsort.so,
built in-tree by build.py).  It mirrors the reference's call shape for the
path -- sort every segment of a device key array (and the values that move
with the keys) given a segment-offset array, in place -- as
cub::DeviceSegmentedRadixSort::SortPairs(keys, vals, n, nseg, d_seg, d_seg+1)
(src/radixseg.cu:121-124) and bb_segsort(keys_d, vals_d, n, d_segs, nseg)
(src/bb_segsort/bb_segsort.h:35-36) do.

Device memory and streams come from PyTorch (plumbing only): the functions
take CUDA tensors and pass their raw device pointers and the current CUDA
stream to the C ABI.  There is no CPU path: if libsegsort.so is missing the
import of `lib()` raises, and every call goes to the GPU kernels.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libsegsort.so"

SEGSORT_OK = 0
SEGSORT_ERR_INVALID_ARG = -1
SEGSORT_ERR_CUDA = -2
SEGSORT_ERR_TIMEOUT = -3
SEGSORT_ERR_NO_MEMORY = -4
SEGSORT_ERR_TOO_LARGE = -5
SEGSORT_ERR_WORKSPACE = -6
SEGSORT_NOALLOC_MAX_N = 1 << 20  # include/segsort.h

# Run-time parameters (SEGSORT_PARAM_* of include/segsort.h).
PARAM_RADIX_MIN_32 = 1
PARAM_RADIX_MIN_64 = 2
PARAM_STREAM_MAX_AVG = 3
PARAM_BUCKET_MIN_AVG = 4
PARAM_MSD = 5
PARAM_TINY_MAX_AVG = 6

KEY_TYPES = ("u32", "i32", "f32", "u64")
KEY_TYPE_CODES = {"u32": 0, "i32": 1, "f32": 2, "u64": 3}  # SEGSORT_KEY_* of include/segsort.h


class BatchItem(ctypes.Structure):
    """segsort_batch_item of include/segsort.h."""
    _fields_ = [("key_type", ctypes.c_int32), ("heads", ctypes.c_int32),
                ("d_keys", ctypes.c_void_p), ("d_vals", ctypes.c_void_p),
                ("n", ctypes.c_int64), ("d_offsets", ctypes.c_void_p),
                ("nseg", ctypes.c_int32), ("reserved", ctypes.c_int32)]

class ServerStats(ctypes.Structure):
    """segsort_server_stats of include/segsort.h."""
    _fields_ = [("requests", ctypes.c_int64), ("batches", ctypes.c_int64),
                ("keys", ctypes.c_int64), ("max_batch", ctypes.c_int64),
                ("peak_bytes", ctypes.c_int64), ("budget_waits", ctypes.c_int64),
                ("status", ctypes.c_int32), ("reserved", ctypes.c_int32)]


# Every symbol include/segsort.h declares, with its ctypes signature.
_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_I32 = ctypes.c_int32
SIGNATURES = {
    **{f"segsort_keys_{t}": ([_P, _I64, _P, _I32, _P], ctypes.c_int) for t in KEY_TYPES},
    **{f"segsort_pairs_{t}": ([_P, _P, _I64, _P, _I32, _P], ctypes.c_int) for t in KEY_TYPES},
    "segsort_pairs_u32_heads": ([_P, _P, _I64, _P, _I32, _P], ctypes.c_int),
    "segsort_keys_u32_heads": ([_P, _I64, _P, _I32, _P], ctypes.c_int),
    "segsort_workspace_bytes": ([_I64, _I32, ctypes.c_int, ctypes.c_int], ctypes.c_size_t),
    "segsort_pairs_u32_ws": ([_P, _P, _I64, _P, _I32, _P, ctypes.c_size_t, _P], ctypes.c_int),
    "segsort_keys_u32_ws": ([_P, _I64, _P, _I32, _P, ctypes.c_size_t, _P], ctypes.c_int),
    "segsort_pairs_u32_noalloc": ([_P, _P, _I64, _P, _I32, _P], ctypes.c_int),
    **{f"segsort_pairs_{t}_desc": ([_P, _P, _I64, _P, _I32, _P], ctypes.c_int) for t in KEY_TYPES},
    "segsort_keys_u32_desc": ([_P, _I64, _P, _I32, _P], ctypes.c_int),
    "segsort_keys_f32_desc": ([_P, _I64, _P, _I32, _P], ctypes.c_int),
    **{f"segsort_pairs_{t}_topk": ([_P, _P, _I64, _P, _I32, _I64, ctypes.c_int, _P, _P, _P, _P],
                                   ctypes.c_int) for t in ("u32", "f32")},
    **{f"segsort_pairs_{t}_v64": ([_P, _P, _I64, _P, _I32, _P], ctypes.c_int) for t in KEY_TYPES},
    "segsort_pairs_u32_reduce_by_key": ([_P, _P, _I64, _P, _I32, _P, _P, _P, _P, _P], ctypes.c_int),
    "segsort_pairs_batch": ([ctypes.POINTER(BatchItem), _I32, _P], ctypes.c_int),
    "segsort_batch_plan_create": ([ctypes.POINTER(BatchItem), _I32, ctypes.POINTER(_P)], ctypes.c_int),
    "segsort_batch_plan_launch": ([_P, _P], ctypes.c_int),
    "segsort_batch_plan_tune": ([_P, _P, ctypes.c_char_p, ctypes.POINTER(_I32)], ctypes.c_int),
    "segsort_batch_plan_workspace_bytes": ([_P], ctypes.c_size_t),
    "segsort_batch_plan_destroy": ([_P], None),
    "segsort_batch_workspace_bytes": ([ctypes.POINTER(BatchItem), _I32], ctypes.c_size_t),
    "segsort_server_create": ([ctypes.c_size_t, _I64, _I32, _I32, ctypes.POINTER(_P)], ctypes.c_int),
    "segsort_server_submit": ([_P, _P, _P, _I64, _P, _I32, _P, _P, ctypes.POINTER(ctypes.c_uint64)],
                              ctypes.c_int),
    "segsort_server_wait": ([_P, ctypes.c_uint64, ctypes.POINTER(ctypes.c_double)], ctypes.c_int),
    "segsort_server_drain": ([_P], ctypes.c_int),
    "segsort_server_get_stats": ([_P, ctypes.POINTER(ServerStats)], ctypes.c_int),
    "segsort_server_destroy": ([_P], None),
    "segsort_pool_bytes": ([ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_uint64)], ctypes.c_int),
    "segsort_set_param": ([ctypes.c_int, _I64], ctypes.c_int),
    "segsort_tune_pairs_u32": ([_P, _P, _I64, _P, _I32, _P, ctypes.c_char_p, ctypes.POINTER(_I64),
                                ctypes.POINTER(_I64), ctypes.POINTER(_I32)], ctypes.c_int),
    "segsort_tune_load": ([ctypes.c_char_p], ctypes.c_int),
    "segsort_tune_clear": ([], None),
    "segsort_tune_lookup": ([ctypes.c_int, _I64, _I32, ctypes.POINTER(_I64), ctypes.POINTER(_I64),
                             ctypes.POINTER(_I32)], ctypes.c_int),
    "segsort_get_param": ([ctypes.c_int, ctypes.POINTER(_I64)], ctypes.c_int),
    "segsort_selftest_wait_timeout": ([ctypes.c_int], ctypes.c_int),
    "segsort_device_status": ([ctypes.c_int], ctypes.c_int),
    "segsort_error_string": ([ctypes.c_int], ctypes.c_char_p),
    "segsort_version": ([], ctypes.c_int),
    "segsort_profile_enable": ([ctypes.c_int], ctypes.c_int),
    "segsort_profile_read": ([ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                              ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                              ctypes.c_int], ctypes.c_int),
}


class SegsortError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        self.code = code
        msg = lib().segsort_error_string(code).decode() if LIB_PATH.exists() else str(code)
        super().__init__(f"{what}: {msg} ({code})" if what else f"{msg} ({code})")


_lib = None


def lib() -> ctypes.CDLL:
    """The loaded C-ABI library.  Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: run build.py (or __graft_entry__.build())")
        L = ctypes.CDLL(str(LIB_PATH))
        for name, (args, res) in SIGNATURES.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def build(verbose: bool = False) -> None:
    from importlib import util
    spec = util.spec_from_file_location("_segsort_build", PKG / "build.py")
    mod = util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build(verbose=verbose)


# ---------------------------------------------------------------------------
# Torch-tensor convenience layer.
# ---------------------------------------------------------------------------
def _key_suffix(t) -> str:
    import torch
    m = {torch.int32: "i32", torch.float32: "f32", torch.int64: "u64"}
    if t.dtype in m:
        return m[t.dtype]
    if hasattr(torch, "uint32") and t.dtype == torch.uint32:
        return "u32"
    if hasattr(torch, "uint64") and t.dtype == torch.uint64:
        return "u64"
    raise TypeError(f"unsupported key dtype {t.dtype}")


def _stream_ptr(stream) -> int:
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def _check(rc: int, what: str) -> None:
    if rc != SEGSORT_OK:
        raise SegsortError(rc, what)


def segsort(keys, offsets, values=None, *, key_type: str | None = None, heads: bool = False,
            stream=None) -> None:
    """Sort every segment of `keys` (and `values`) in place on the GPU.

    keys     CUDA tensor, contiguous; its dtype picks the key type unless
             `key_type` ("u32", "i32", "f32", "u64") reinterprets its bits
             (e.g. an int32 tensor holding uint32 keys with key_type="u32").
    offsets  CUDA int32 tensor: nseg+1 CSR offsets, or nseg heads with heads=True.
    values   optional CUDA tensor of 32-bit values (uint32 bits) moved with keys.
    """
    if not keys.is_cuda or not offsets.is_cuda:
        raise ValueError("keys and offsets must be CUDA tensors")
    if not keys.is_contiguous() or not offsets.is_contiguous():
        raise ValueError("keys and offsets must be contiguous")
    import torch
    if offsets.dtype != torch.int32:
        raise TypeError("offsets must be int32")
    suf = key_type or _key_suffix(keys)
    n = keys.numel()
    nseg = offsets.numel() - (0 if heads else 1)
    if nseg < 0:
        raise ValueError("offsets must hold nseg+1 entries")
    L = lib()
    st = _stream_ptr(stream)
    if values is None:
        if heads:
            if suf != "u32":
                raise ValueError("heads-only offsets support u32 keys")
            rc = L.segsort_keys_u32_heads(keys.data_ptr(), n, offsets.data_ptr(), nseg, st)
        else:
            rc = getattr(L, f"segsort_keys_{suf}")(keys.data_ptr(), n, offsets.data_ptr(), nseg, st)
    else:
        if values.numel() != n or not values.is_cuda or values.element_size() != 4:
            raise ValueError("values must be a CUDA tensor of n 32-bit elements")
        if heads:
            if suf != "u32":
                raise ValueError("heads-only offsets support u32 keys")
            rc = L.segsort_pairs_u32_heads(keys.data_ptr(), values.data_ptr(), n,
                                           offsets.data_ptr(), nseg, st)
        else:
            rc = getattr(L, f"segsort_pairs_{suf}")(keys.data_ptr(), values.data_ptr(), n,
                                                     offsets.data_ptr(), nseg, st)
    _check(rc, f"segsort_{'pairs' if values is not None else 'keys'}_{suf}")


def device_status(clear: bool = True) -> int:
    """Synchronise and return the device-side status (0 = no bounded wait gave up)."""
    return lib().segsort_device_status(1 if clear else 0)


def get_param(param: int) -> int:
    v = ctypes.c_int64()
    _check(lib().segsort_get_param(param, ctypes.byref(v)), "segsort_get_param")
    return v.value


def set_param(param: int, value: int) -> None:
    _check(lib().segsort_set_param(param, value), "segsort_set_param")


class params:
    """Context manager that sets run-time parameters and restores them:
    `with params({PARAM_RADIX_MIN_32: 1 << 30}): ...`"""

    def __init__(self, values: dict):
        self._values = dict(values)
        self._saved = {}

    def __enter__(self):
        for k, v in self._values.items():
            self._saved[k] = get_param(k)
            set_param(k, v)
        return self

    def __exit__(self, *exc):
        for k, v in self._saved.items():
            set_param(k, v)


def workspace_bytes(n: int, nseg: int, key_bytes: int = 4, val_bytes: int = 4) -> int:
    return lib().segsort_workspace_bytes(n, nseg, key_bytes, val_bytes)


def profile_enable(on: bool = True) -> None:
    lib().segsort_profile_enable(1 if on else 0)


def profile_read(reset: bool = True) -> dict:
    """Phase times (ms) and kernel launch counts accumulated while enabled."""
    t, l = ctypes.c_double(), ctypes.c_double()
    nt, nl = ctypes.c_int64(), ctypes.c_int64()
    _check(lib().segsort_profile_read(ctypes.byref(t), ctypes.byref(l), ctypes.byref(nt),
                                      ctypes.byref(nl), 1 if reset else 0), "profile_read")
    return {"tile_ms": t.value, "large_ms": l.value, "tile_launches": nt.value,
            "large_launches": nl.value}


# ---------------------------------------------------------------------------
# Batched form.
# ---------------------------------------------------------------------------
def batch_items(instances) -> ctypes.Array:
    """ctypes array of segsort_batch_item from (keys, values, offsets, key_type)
    tuples of CUDA tensors (CSR offsets: nseg + 1 int32 entries)."""
    import torch
    arr = (BatchItem * len(instances))()
    for i, (keys, values, offsets, key_type) in enumerate(instances):
        if not (keys.is_cuda and values.is_cuda and offsets.is_cuda):
            raise ValueError("batch tensors must be CUDA tensors")
        if offsets.dtype != torch.int32 or values.element_size() != 4:
            raise TypeError("offsets must be int32 and values 32-bit")
        if values.numel() != keys.numel():
            raise ValueError("values must hold one element per key")
        arr[i] = BatchItem(KEY_TYPE_CODES[key_type], 0, keys.data_ptr(), values.data_ptr(),
                           keys.numel(), offsets.data_ptr(), offsets.numel() - 1, 0)
    return arr


def segsort_batch(instances, stream=None) -> None:
    """Sort every instance of a batch in place with one launch per kernel and key type."""
    items = batch_items(instances)
    _check(lib().segsort_pairs_batch(items, len(items), _stream_ptr(stream)), "segsort_pairs_batch")


class BatchPlan:
    """A batch captured once into a CUDA graph; launch() replays it."""

    def __init__(self, instances):
        self._items = batch_items(instances)
        self._h = ctypes.c_void_p()
        _check(lib().segsort_batch_plan_create(self._items, len(self._items), ctypes.byref(self._h)),
               "segsort_batch_plan_create")

    def launch(self, stream=None) -> None:
        _check(lib().segsort_batch_plan_launch(self._h, _stream_ptr(stream)), "segsort_batch_plan_launch")

    def tune(self, cache_path: str | None = None, stream=None) -> int:
        """Choose the merge passes' launch shape (see segsort_batch_plan_tune);
        returns the chosen CTAs per SM."""
        k = ctypes.c_int32()
        path = None if cache_path is None else str(cache_path).encode()
        _check(lib().segsort_batch_plan_tune(self._h, _stream_ptr(stream), path, ctypes.byref(k)),
               "segsort_batch_plan_tune")
        return k.value

    @property
    def workspace_bytes(self) -> int:
        return lib().segsort_batch_plan_workspace_bytes(self._h)

    def close(self) -> None:
        if self._h:
            lib().segsort_batch_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# Served form.
# ---------------------------------------------------------------------------
class Server:
    """Continuous-batching request server on the current device.

    submit() takes host buffers (numpy arrays or CPU tensors; pinned memory
    lets the copies overlap the sorts) that must stay alive until wait()
    returns for that ticket; results land in keys_out / vals_out."""

    def __init__(self, budget_bytes: int, max_batch: int = 0, depth: int = 0,
                 max_batch_keys: int = 0):
        self._h = ctypes.c_void_p()
        _check(lib().segsort_server_create(budget_bytes, max_batch_keys, max_batch, depth,
                                           ctypes.byref(self._h)), "segsort_server_create")
        self._keep = {}

    @staticmethod
    def _ptr(a) -> int:
        return a.ctypes.data if hasattr(a, "ctypes") else a.data_ptr()

    def submit(self, keys, vals, offsets, keys_out, vals_out) -> int:
        t = ctypes.c_uint64()
        n = len(keys)
        _check(lib().segsort_server_submit(self._h, self._ptr(keys), self._ptr(vals), n,
                                           self._ptr(offsets), len(offsets) - 1,
                                           self._ptr(keys_out), self._ptr(vals_out),
                                           ctypes.byref(t)), "segsort_server_submit")
        self._keep[t.value] = (keys, vals, offsets, keys_out, vals_out)
        return t.value

    def wait(self, ticket: int) -> float:
        ms = ctypes.c_double()
        rc = lib().segsort_server_wait(self._h, ticket, ctypes.byref(ms))
        self._keep.pop(ticket, None)
        _check(rc, "segsort_server_wait")
        return ms.value

    def drain(self) -> None:
        _check(lib().segsort_server_drain(self._h), "segsort_server_drain")

    def stats(self) -> dict:
        st = ServerStats()
        _check(lib().segsort_server_get_stats(self._h, ctypes.byref(st)), "segsort_server_get_stats")
        return {f: getattr(st, f) for f, _ in ServerStats._fields_ if f != "reserved"}

    def close(self) -> None:
        if self._h:
            lib().segsort_server_destroy(self._h)
            self._h = ctypes.c_void_p()
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
