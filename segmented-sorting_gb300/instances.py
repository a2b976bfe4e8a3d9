"""Seeded synthetic instances for the segmented sort (numpy, host side).

Every value is a function of (seed, index) through splitmix64, the same
counter-based stream csrc/gen_instance.cpp uses, so instances are identical
on every machine and between the Python and C++ generators (lognormal
lengths go through floating-point exp/log/cos and may differ by one in rare
rounding cases; keys and equal/diff offsets are exact integer arithmetic).

Workloads (the reference's sweep shapes, scripts/genequalseg.sh:3-16, and
the benchmark configurations built on them):
  equal_offsets      n / len equal segments (utils/gen_equal.cpp:13-16)
  diff_offsets       nseg random distinct cut points (utils/gen_diff.cpp:11-42)
  lognormal_offsets  lognormal(mu, sigma) lengths clipped to [1, max], summed
                     to n, the last one truncated, plus ~empty_frac empty ones
  uniform_keys       keys uniform in [0, 2^bits)
  zipf_keys          Zipf(a) ranks via the inverse CDF of the continuous power
                     law, truncated to uint32 (heavily repeated small keys)
"""
from __future__ import annotations

import numpy as np

_GOLD = np.uint64(0x9E3779B97F4A7C15)
_LANE = np.uint64(0xD1B54A32D192ED03)


def splitmix64(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        x = x.astype(np.uint64) + _GOLD
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return x ^ (x >> np.uint64(31))


def draw(seed: int, lane: int, start: int, count: int) -> np.ndarray:
    """Values start..start+count-1 of the counter-based stream (seed, lane)."""
    with np.errstate(over="ignore"):
        base = np.uint64(seed) * _GOLD + np.uint64(lane) * _LANE + np.uint64(start + 1)
        return splitmix64(base + np.arange(count, dtype=np.uint64))


def _unit(r: np.ndarray) -> np.ndarray:
    return ((r >> np.uint64(11)).astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)


def uniform_keys(n: int, seed: int = 1, bits: int = 32, dtype=np.uint32) -> np.ndarray:
    """Keys uniform in [0, 2^bits): the top `bits` bits of the stream."""
    r = draw(seed, 0, 0, n)
    if bits < 64:
        r = r >> np.uint64(64 - bits)
    return r.astype(dtype)


def zipf_keys(n: int, seed: int = 1, a: float = 1.1) -> np.ndarray:
    u = _unit(draw(seed, 5, 0, n))
    with np.errstate(over="ignore"):
        r = np.floor(u ** (-1.0 / (a - 1.0)))
    return np.minimum(r, 4294967295.0).astype(np.uint32)


def equal_offsets(n: int, length: int) -> np.ndarray:
    nseg = n // length
    return (np.arange(nseg + 1, dtype=np.int64) * length).astype(np.int32)


def diff_offsets(n: int, nseg: int, seed: int = 1) -> np.ndarray:
    """nseg segments cut at nseg-1 distinct random points of [1, n), sorted."""
    if nseg < 1 or nseg > n:
        raise ValueError("need 1 <= nseg <= n")
    taken = np.zeros(n, dtype=bool)
    taken[0] = True
    cuts = [0]
    i = 0
    while len(cuts) < nseg:
        need = nseg - len(cuts)
        r = (draw(seed, 1, i, 2 * need + 16) % np.uint64(n)).astype(np.int64)
        i += len(r)
        for x in r:
            if not taken[x]:
                taken[x] = True
                cuts.append(int(x))
                if len(cuts) == nseg:
                    break
    return np.concatenate([np.sort(np.array(cuts, dtype=np.int64)), [n]]).astype(np.int32)


def lognormal_offsets(n: int, seed: int = 1, mu: float = 4.0, sigma: float = 2.5,
                      max_len: int = 1 << 22, empty_frac: float = 0.01) -> np.ndarray:
    lens = []
    total = 0
    i = 0
    while total < n:
        m = 4096
        u = _unit(draw(seed, 2, 2 * i, 2 * m))
        u1, u2 = u[0::2], u[1::2]
        z = np.sqrt(-2.0 * np.log(u1)) * np.cos(6.283185307179586 * u2)
        ln = np.clip(np.rint(np.exp(mu + sigma * z)), 1, max_len).astype(np.int64)
        for x in ln:
            x = min(int(x), n - total)
            lens.append(x)
            total += x
            if total >= n:
                break
        i += m
    lens = np.array(lens, dtype=np.int64)
    ends = np.cumsum(lens)
    empty = _unit(draw(seed, 3, 0, len(lens))) < empty_frac
    # segment i is followed by an empty segment when empty[i]
    reps = np.where(empty, 2, 1)
    off = np.concatenate([[0], np.repeat(ends, reps)])
    return off.astype(np.int32)


def equal_offsets_ragged(n: int, length: int) -> np.ndarray:
    """n // length equal segments and, when length does not divide n, one
    shorter last segment, so every element is in a segment."""
    off = equal_offsets(n, length).astype(np.int64)
    if off[-1] < n:
        off = np.concatenate([off, [n]])
    return off.astype(np.int32)


def typed_keys(n: int, seed: int, key_type: str) -> np.ndarray:
    """Keys of a batch instance: u32 / i32 / u64 uniform over the type's
    range, f32 uniform in [-1000, 1000) (both signs, no NaN)."""
    if key_type == "u32":
        return uniform_keys(n, seed, 32)
    if key_type == "i32":
        return uniform_keys(n, seed, 32).view(np.int32)
    if key_type == "u64":
        return uniform_keys(n, seed, 64, np.uint64)
    if key_type == "f32":
        return ((_unit(draw(seed, 0, 0, n)) * 2.0 - 1.0) * 1000.0).astype(np.float32)
    raise ValueError(key_type)


BATCH_KEY_TYPES = ("u32", "u64", "f32")


def batch_specs(count: int = 64, seed: int = 4, lo_log: float = 16, hi_log: float = 24,
                key_types=BATCH_KEY_TYPES) -> list[dict]:
    """Shapes of the mixed batch: n log-uniform in [2^lo_log, 2^hi_log];
    segment lengths equal (length log-uniform in [2, 2^16], ragged last
    segment) or lognormal as in the uneven workload, each with probability
    1/2; key types cycle through key_types."""
    u = _unit(draw(seed, 6, 0, 3 * count))
    specs = []
    for i in range(count):
        n = int(round(2.0 ** (lo_log + (hi_log - lo_log) * u[3 * i])))
        specs.append({
            "n": n,
            "dist": "equal" if u[3 * i + 1] < 0.5 else "lognormal",
            "length": int(round(2.0 ** (1 + 15 * u[3 * i + 2]))),
            "key_type": key_types[i % len(key_types)],
            "seed": seed * 1000 + i,
        })
    return specs


def batch_offsets(spec: dict) -> np.ndarray:
    """Offsets of one batch instance."""
    n = spec["n"]
    if spec["dist"] == "equal":
        return equal_offsets_ragged(n, spec["length"])
    return lognormal_offsets(n, spec["seed"])


def batch_instance(spec: dict):
    """(offsets, keys) of one batch instance."""
    return batch_offsets(spec), typed_keys(spec["n"], spec["seed"], spec["key_type"])


# ---------------------------------------------------------------------------
# Binary instance format (segsort_driver.exe reads it, gen_instance.exe
# --binary writes it): 32-byte header {b"SGSB", version 1, key bytes (4/8),
# key kind (0 unsigned, 1 signed, 2 float), nseg, n}, nseg+1 int32 offsets,
# zero padding to a multiple of 8 bytes, n little-endian keys.
_KIND = {np.dtype(np.uint32): (4, 0), np.dtype(np.int32): (4, 1),
         np.dtype(np.float32): (4, 2), np.dtype(np.uint64): (8, 0)}


def write_binary_instance(offsets: np.ndarray, keys: np.ndarray) -> bytes:
    kb, kind = _KIND[keys.dtype]
    head = np.array([1, kb, kind], dtype="<u4").tobytes()
    counts = np.array([len(offsets) - 1, len(keys)], dtype="<u8").tobytes()
    off = np.asarray(offsets, dtype="<i4").tobytes()
    pad = b"\0" * ((8 - (32 + len(off)) % 8) % 8)
    return b"SGSB" + head + counts + off + pad + keys.astype(keys.dtype.newbyteorder("<")).tobytes()


def read_binary_instance(data: bytes):
    """(offsets, keys) of a binary instance."""
    if data[:4] != b"SGSB":
        raise ValueError("not a binary instance")
    version, kb, kind = np.frombuffer(data, dtype="<u4", count=3, offset=4)
    nseg, n = (int(x) for x in np.frombuffer(data, dtype="<u8", count=2, offset=16))
    if version != 1:
        raise ValueError("unknown version")
    off = np.frombuffer(data, dtype="<i4", count=nseg + 1, offset=32).astype(np.int32)
    at = (32 + 4 * (nseg + 1) + 7) // 8 * 8
    dt = {(4, 0): np.uint32, (4, 1): np.int32, (4, 2): np.float32, (8, 0): np.uint64}[(int(kb), int(kind))]
    keys = np.frombuffer(data, dtype=np.dtype(dt).newbyteorder("<"), count=n, offset=at).astype(dt)
    return off, keys


def instance(workload: str, n: int, seed: int = 1, length: int = 0, nseg: int = 0,
             bits: int = 32):
    """(offsets, keys) of a named workload."""
    if workload == "equal":
        return equal_offsets(n, length), uniform_keys(n, seed, bits)
    if workload == "diff":
        return diff_offsets(n, nseg, seed), uniform_keys(n, seed, bits)
    if workload == "lognormal":
        return lognormal_offsets(n, seed), uniform_keys(n, seed, bits)
    if workload == "lognormal-zipf":
        return lognormal_offsets(n, seed), zipf_keys(n, seed)
    raise ValueError(workload)


# ---------------------------------------------------------------------------
# Device-side generation (torch int64 arithmetic wraps like uint64; logical
# shifts are emulated with masks).  Produces exactly uniform_keys(n, seed, bits).
def _s64(x: int) -> int:
    x &= (1 << 64) - 1
    return x - (1 << 64) if x >= (1 << 63) else x


def _srl(t, k: int):
    return (t >> k) & ((1 << (64 - k)) - 1)


def device_draw(n: int, seed: int, lane: int = 0, device="cuda"):
    """int64 CUDA tensor holding the bits of draw(seed, lane, 0, n)."""
    import torch
    base = _s64(seed * 0x9E3779B97F4A7C15 + lane * 0xD1B54A32D192ED03 + 1)
    x = torch.arange(n, dtype=torch.int64, device=device) + base
    x = x + _s64(0x9E3779B97F4A7C15)
    x = (x ^ _srl(x, 30)) * _s64(0xBF58476D1CE4E5B9)
    x = (x ^ _srl(x, 27)) * _s64(0x94D049BB133111EB)
    return x ^ _srl(x, 31)


def device_uniform_keys(n: int, seed: int = 1, bits: int = 32, device="cuda"):
    """int32 CUDA tensor holding the uint32 bits of uniform_keys(n, seed, bits)."""
    import torch
    k = _srl(device_draw(n, seed, 0, device), 64 - bits)
    return (k - (k >= (1 << 31)).to(torch.int64) * (1 << 32)).to(torch.int32)


def device_typed_keys(n: int, seed: int, key_type: str, device="cuda"):
    """CUDA tensor with the bits of typed_keys(n, seed, key_type): int32 for
    u32/i32, float32 for f32, int64 for u64."""
    import torch
    if key_type in ("u32", "i32"):
        return device_uniform_keys(n, seed, 32, device)
    x = device_draw(n, seed, 0, device)
    if key_type == "u64":
        return x
    if key_type == "f32":
        u = (_srl(x, 11).to(torch.float64) + 0.5) * (1.0 / 9007199254740992.0)
        return ((u * 2.0 - 1.0) * 1000.0).to(torch.float32)
    raise ValueError(key_type)
