#!/usr/bin/env python3
"""Benchmark of the GB300 segmented sort on its headline workload.

Workload (one "step"): the equal-segment sweep -- for every segment length
2^1 .. 2^20, one instance of n = 2^24 uint32 keys uniform in [0, 2^32) with
uint32 values = input index, split into n / len equal segments, sorted in
place through the library's C ABI (segsort_pairs_u32).  Every step sorts
fresh copies (inputs created before the timed region, each instance 128 MiB,
so consecutive calls never find their input in the 126 MB L2).

Printed JSON line (rank 0):
  value       Gkeys/s over the K timed steps, inputs resident in HBM
  e2e         the same through the Python API with pinned host buffers:
              host->device copy of keys+values, sort, device->host copy,
              four instances in flight on four streams; every instance read
              back is checked (sorted within segments, keys moved with their
              values)
  roofline    the dominant kernel, algorithmic bytes (read and write every
              key and value once per pass over them, plus the offsets or the
              radix digit counts) / its CUDA-event time measured live on the
              launching stream, against the measured HBM copy bandwidth
  cpu_baseline  the oracle's per-segment std::stable_sort (the reference's
              CPU algorithm, src/mseq.cu:44-49) on the same full instances:
              one step on all host threads and one on a single thread (the
              reference's mseq is sequential)
  per_len     per segment length: ms, Gkeys/s, fraction of the HBM roofline and route
  batched, served, configs   the other workloads (64-instance batch, Poisson
              request stream, 2^20 keys-only, 2^25 lognormal, low entropy)

--impl reference times that CPU algorithm as the reference arm (rank 0), on
the same instances and the same config.  --served-only runs the request
stream alone (e.g. the full 1k..50k req/s sweep).
"""
from __future__ import annotations

import argparse
import ctypes
import importlib
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import __graft_entry__ as entry  # noqa: E402

METRIC = "segsort Gkeys/s vs segment size, % HBM roofline; batched/served p50/p99 ms"
WORKLOAD = ("equal-segment sweep: 2^24 uint32 key/value pairs per instance, keys uniform "
            "in [0,2^32), values = index, segment length 2^1..2^20 (one instance each)")
BYTES_PER_PAIR = 16  # read key+value once, write key+value once


def max_over_ranks(x: float, world: int, device=None) -> float:
    """The largest x over the job's ranks (x itself for one rank): the
    timed region of a multi-rank run is its slowest rank's."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_gkeys(keys_per_step: int, steps: int, world: int, ms: float) -> float:
    """Whole-job throughput: the keys every rank sorted (each rank sorts its
    own replica of the workload) over the slowest rank's time."""
    return keys_per_step * steps * world / (ms * 1e-3) / 1e9
FALLBACK_HBM_GBS = 6800.0


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--log-n", type=int, default=24)
    p.add_argument("--lengths", type=str, default="1-20",
                   help="log2 segment lengths, e.g. 1-20 or 4,8,12")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-batched", action="store_true", help="skip the 64-instance batch")
    p.add_argument("--no-configs", action="store_true", help="skip the other workloads")
    p.add_argument("--no-served", action="store_true", help="skip the served-form stream")
    p.add_argument("--served-requests", type=int, default=100000)
    p.add_argument("--served-rates", type=str, default="5000,10000,50000")
    p.add_argument("--served-only", action="store_true",
                   help="run only the served-form request stream and print its JSON")
    return p.parse_args()


def log_lengths(spec: str) -> list[int]:
    out = []
    for part in spec.split(","):
        if "-" in part:
            a, b = part.split("-")
            out.extend(range(int(a), int(b) + 1))
        else:
            out.append(int(part))
    return out


def peak_hbm() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def traffic_per_launch() -> dict | None:
    """DRAM bytes per launch of the profiled kernels, from the committed ncu
    summary (profiles/traffic.json); None until one is committed."""
    p = ROOT / "profiles" / "traffic.json"
    try:
        return json.loads(p.read_text())
    except Exception:
        return None


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while running."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id: str | None):
        self.gpu_id = gpu_id
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                   "-lms", "50"]
            if self.gpu_id:
                cmd += ["-i", self.gpu_id]
            self.proc = subprocess.Popen(cmd, stdout=open(self.path, "w"),
                                         stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.1)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 8:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[4 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


# ---------------------------------------------------------------------------
def bench_config(n: int, lengths: list[int], world: int) -> dict:
    """The workload's config, identical for both arms.  The default run is
    WORKLOAD; other sizes and length lists are named by what they are."""
    log_n = n.bit_length() - 1
    if n == 1 << 24 and lengths == list(range(1, 21)):
        workload = WORKLOAD
    else:
        span = (f"2^{lengths[0]}..2^{lengths[-1]}" if lengths == list(range(lengths[0], lengths[-1] + 1))
                else ", ".join(f"2^{x}" for x in lengths))
        workload = (f"equal-segment sweep: 2^{log_n} uint32 key/value pairs per instance, keys "
                    f"uniform in [0,2^32), values = index, segment length {span} (one instance each)")
    mib = 8 * n / 2**20
    l2 = (f"inputs larger than L2: {mib:g} MiB fresh instance per call" if 8 * n > 129e6
          else f"inputs smaller than L2 ({mib:g} MiB fresh instance per call)")
    return {"workload": workload, "n": n, "log2_lengths": lengths, "l2": l2,
            "parallelism": f"replicas{world}"}


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.machine()


class CpuSweep:
    """The sweep's instances in host memory (the same keys the GPU arm
    sorts), sorted by the oracle's std::stable_sort per segment -- the
    reference's mseq algorithm -- on fresh copies every step."""

    def __init__(self, O, inst, n: int, lengths: list[int]):
        self.O, self.n = O, n
        self.items = [(inst.uniform_keys(n, seed=1000 + lg, bits=32), inst.equal_offsets(n, 1 << lg))
                      for lg in lengths]
        self.vals = np.arange(n, dtype=np.uint32)
        self.k = np.empty(n, np.uint32)
        self.v = np.empty(n, np.uint32)

    def step(self, threads: int) -> float:
        """Seconds spent sorting (copies outside)."""
        total = 0.0
        kp = self.k.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
        vp = self.v.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
        for keys, off in self.items:
            np.copyto(self.k, keys)
            np.copyto(self.v, self.vals)
            op = off.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
            t0 = time.perf_counter()
            self.O.lib().oracle_segsort_pairs_u32(kp, vp, self.n, op, len(off) - 1, threads)
            total += time.perf_counter() - t0
        return total

    @property
    def keys_per_step(self) -> int:
        return self.n * len(self.items)


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    entry.load_package()
    inst = importlib.import_module(f"{entry.PKG_NAME}.instances")
    lengths = log_lengths(args.lengths)
    n = 1 << args.log_n
    threads = O.default_threads()
    sweep = CpuSweep(O, inst, n, lengths)
    for _ in range(args.warmup):
        sweep.step(threads)
    secs = sum(sweep.step(threads) for _ in range(args.steps))
    value = sweep.keys_per_step * args.steps / secs / 1e9
    sample = (f"the full sweep every step: {len(lengths)} instances of {n} pairs, "
              f"std::stable_sort per segment on {threads} threads")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Gkeys/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": secs / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": bench_config(n, lengths, world),
        "cpu_baseline": {"value": value, "unit": "Gkeys/s", "cores": threads, "kind": "port",
                         "cpu_model": cpu_model(), "sample": sample},
        "e2e": {"value": value, "unit": "Gkeys/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }), flush=True)


# ---------------------------------------------------------------------------
BATCH_WORKLOAD = ("64 independent instances, n log-uniform in [2^16, 2^24], segment lengths "
                  "equal (length log-uniform in [2, 2^16]) or lognormal(4, 2.5), keys u32/u64/f32 "
                  "in turn, uint32 values = index")
_TORCH_KEY = {"u32": "int32", "i32": "int32", "f32": "float32", "u64": "int64"}


def _timed(stream, fn, restore, warmup: int, steps: int) -> list[float]:
    """CUDA-event ms of fn() per step; restore() (untimed) refreshes the inputs."""
    import torch
    out = []
    for s in range(warmup + steps):
        restore()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        if s >= warmup:
            out.append((a, b))
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in out]


def bench_batched(pkg, inst, dev, stream, warmup: int, steps: int) -> dict:
    """The 64-instance mixed batch: one replay of a batch plan (one CUDA graph)
    against the same 64 instances as back-to-back plain calls, on fresh copies
    of the inputs every step (1.7 GB of pairs: above L2)."""
    import torch
    L = pkg.lib()
    st = stream.cuda_stream
    specs = inst.batch_specs()
    rows = []
    for s in specs:
        off = torch.from_numpy(inst.batch_offsets(s)).to(dev)
        keys = inst.device_typed_keys(s["n"], s["seed"], s["key_type"], device=dev)
        vals = torch.arange(s["n"], dtype=torch.int32, device=dev)
        rows.append({"spec": s, "off": off, "k0": keys, "v0": vals,
                     "k": torch.empty_like(keys), "v": torch.empty_like(vals)})
    total = sum(s["n"] for s in specs)

    def restore():
        for r in rows:
            r["k"].copy_(r["k0"])
            r["v"].copy_(r["v0"])

    def plain():
        for r in rows:
            s = r["spec"]
            rc = getattr(L, f"segsort_pairs_{s['key_type']}")(
                r["k"].data_ptr(), r["v"].data_ptr(), s["n"], r["off"].data_ptr(),
                r["off"].numel() - 1, st)
            if rc != 0:
                raise pkg.SegsortError(rc, "plain call")

    items = (pkg.BatchItem * len(rows))(*[
        pkg.BatchItem(pkg.KEY_TYPE_CODES[r["spec"]["key_type"]], 0, r["k"].data_ptr(),
                      r["v"].data_ptr(), r["spec"]["n"], r["off"].data_ptr(),
                      r["off"].numel() - 1, 0) for r in rows])

    def one_shot():
        rc = L.segsort_pairs_batch(items, len(rows), st)
        if rc != 0:
            raise pkg.SegsortError(rc, "segsort_pairs_batch")

    plan = ctypes.c_void_p()
    rc = L.segsort_batch_plan_create(items, len(rows), ctypes.byref(plan))
    if rc != 0:
        raise pkg.SegsortError(rc, "segsort_batch_plan_create")
    # Autotuner: the merge passes' launch shape for this batch, measured on
    # its own data (no cache file: always measured here).
    tuned = ctypes.c_int32()
    restore()
    rc = L.segsort_batch_plan_tune(plan, st, None, ctypes.byref(tuned))
    if rc != 0:
        raise pkg.SegsortError(rc, "segsort_batch_plan_tune")

    def replay():
        rc = L.segsort_batch_plan_launch(plan, st)
        if rc != 0:
            raise pkg.SegsortError(rc, "segsort_batch_plan_launch")

    def group_times() -> dict:
        """Per key type: a plan of that type's instances alone, and the same
        instances as plain calls (median ms)."""
        out = {}
        for kt in sorted({r["spec"]["key_type"] for r in rows}):
            sub = [i for i, r in enumerate(rows) if r["spec"]["key_type"] == kt]
            sub_items = (pkg.BatchItem * len(sub))(*[items[i] for i in sub])
            gp = ctypes.c_void_p()
            if L.segsort_batch_plan_create(sub_items, len(sub), ctypes.byref(gp)) != 0:
                continue
            try:
                t_g = _timed(stream, lambda: L.segsort_batch_plan_launch(gp, st), restore, 1, 3)
            finally:
                L.segsort_batch_plan_destroy(gp)

            def plain_sub():
                for i in sub:
                    r, sp = rows[i], rows[i]["spec"]
                    getattr(L, f"segsort_pairs_{sp['key_type']}")(
                        r["k"].data_ptr(), r["v"].data_ptr(), sp["n"], r["off"].data_ptr(),
                        r["off"].numel() - 1, st)
            t_p = _timed(stream, plain_sub, restore, 1, 3)
            keys = sum(rows[i]["spec"]["n"] for i in sub)
            out[kt] = {"instances": len(sub), "keys": keys,
                       "plan_ms": round(statistics.median(t_g), 4),
                       "plain_ms": round(statistics.median(t_p), 4)}
        return out

    def plain_launches() -> int:
        """Kernels one pass of plain calls launches (the library's phase
        records: tile-sort and long-segment launches of every call)."""
        pkg.profile_enable(True)
        pkg.profile_read(reset=True)
        restore()
        plain()
        torch.cuda.synchronize()
        p = pkg.profile_read(reset=True)
        pkg.profile_enable(False)
        return int(p["tile_launches"] + p["large_launches"])

    try:
        n_plain_launches = plain_launches()
        t_plain = _timed(stream, plain, restore, warmup, steps)
        ref = [(r["k"].clone(), r["v"].clone()) for r in rows]
        t_one = _timed(stream, one_shot, restore, warmup, steps)
        t_plan = _timed(stream, replay, restore, warmup, steps)
        identical = all(torch.equal(r["k"], k) and torch.equal(r["v"], v)
                        for r, (k, v) in zip(rows, ref))
        ws = L.segsort_batch_plan_workspace_bytes(plan)
        groups = group_times()
    finally:
        L.segsort_batch_plan_destroy(plan)
    if pkg.device_status() != 0:
        raise RuntimeError("device status reports a bounded wait that gave up")
    if not identical:
        raise RuntimeError("batched output differs from the plain calls")
    med = {k: statistics.median(v) for k, v in
           (("plain", t_plain), ("one_shot", t_one), ("plan", t_plan))}
    types = sorted({s["key_type"] for s in specs})
    return {
        "workload": BATCH_WORKLOAD, "instances": len(specs), "keys": total,
        "key_types": {t: sum(1 for s in specs if s["key_type"] == t) for t in types},
        "plain_ms": round(med["plain"], 4), "one_shot_ms": round(med["one_shot"], 4),
        "plan_ms": round(med["plan"], 4),
        "plain_gkeys_s": round(total / (med["plain"] * 1e-3) / 1e9, 3),
        "plan_gkeys_s": round(total / (med["plan"] * 1e-3) / 1e9, 3),
        "speedup_plan_vs_plain": round(med["plain"] / med["plan"], 3),
        "plan_p99_ms": round(float(np.percentile(t_plan, 99)), 4),
        "identical_to_plain": identical, "plan_workspace_bytes": ws, "steps": steps,
        "tuned_merge_ctas_per_sm": tuned.value, "by_key_type": groups,
        # per key-type group: classify, the bucket kernel, the list kernel,
        # the long-segment kernel
        "launches": {"plain": n_plain_launches, "plan_graph": 4 * len(types)},
    }


SERVED_WORKLOAD = ("Poisson request stream, seed 7; each request a uint32 key/value sort with "
                   "n log-uniform in [2^10, 2^24] and lognormal(4, 2.5) segment lengths (1% empty); "
                   "64 GB HBM admission budget; inputs and outputs in pinned host memory")


def bench_served(requests: int, rates: str) -> dict:
    """The served form against the one-request-per-call loop, through the
    native driver serve_bench.exe (one JSON line per arrival rate)."""
    exe = entry.PKG_DIR / "serve_bench.exe"
    cmd = [str(exe), "--requests", str(requests), "--rates", rates, "--budget-gb", "64",
           "--seed", "7"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=3600)
    if r.returncode != 0:
        raise RuntimeError(f"serve_bench failed ({r.returncode}): {r.stderr[-2000:]}")
    rows = [json.loads(line) for line in r.stdout.splitlines() if line.strip()]
    return {"workload": SERVED_WORKLOAD,
            "sample": f"{requests} requests per rate (the same requests at every rate), "
                      f"rates {rates} req/s",
            "requests": requests, "rates": rows}


def bench_configs(pkg, inst, dev, stream, warmup: int, steps: int) -> dict:
    """The plain call on the other single-instance workloads: 2^20 keys-only
    (1024 x 1024, keys < 2^31), 2^25 pairs with lognormal segment lengths
    (uniform and Zipf(1.1) keys), and the equal-segment sweep's low-entropy
    variant (2^24 pairs, keys in [0, 16), segment lengths 2^1..2^20)."""
    import torch
    L = pkg.lib()
    st = stream.cuda_stream
    out = {}
    n1 = 1 << 20
    k0 = inst.device_uniform_keys(n1, seed=1, bits=31, device=dev)
    o1 = torch.from_numpy(inst.equal_offsets(n1, 1024)).to(dev)
    k = torch.empty_like(k0)
    t = _timed(stream, lambda: L.segsort_keys_u32(k.data_ptr(), n1, o1.data_ptr(), 1024, st),
               lambda: k.copy_(k0), warmup, steps)
    ms = statistics.median(t)
    out["keys_2e20_1024x1024"] = {"ms": round(ms, 5), "gkeys_s": round(n1 / (ms * 1e-3) / 1e9, 3)}
    n3 = 1 << 25
    o3n = inst.lognormal_offsets(n3, seed=1)
    o3 = torch.from_numpy(o3n).to(dev)
    lens = np.diff(o3n)
    v0 = torch.arange(n3, dtype=torch.int32, device=dev)
    for name, keys in (("uniform", inst.device_uniform_keys(n3, seed=1, bits=32, device=dev)),
                       ("zipf", torch.from_numpy(inst.zipf_keys(n3, seed=1).view(np.int32)).to(dev))):
        kk, vv = torch.empty_like(keys), torch.empty_like(v0)

        def restore():
            kk.copy_(keys)
            vv.copy_(v0)

        t = _timed(stream, lambda: L.segsort_pairs_u32(kk.data_ptr(), vv.data_ptr(), n3,
                                                       o3.data_ptr(), len(o3n) - 1, st),
                   restore, warmup, steps)
        ms = statistics.median(t)
        out[f"pairs_2e25_lognormal_{name}"] = {
            "ms": round(ms, 4), "gkeys_s": round(n3 / (ms * 1e-3) / 1e9, 3),
            "segments": int(len(lens)), "empty": int((lens == 0).sum()),
            "max_len": int(lens.max())}
    n2 = 1 << 24
    k4 = inst.device_uniform_keys(n2, seed=16, bits=4, device=dev)
    v2 = torch.arange(n2, dtype=torch.int32, device=dev)
    kk, vv = torch.empty_like(k4), torch.empty_like(v2)

    def restore4():
        kk.copy_(k4)
        vv.copy_(v2)

    per = {}
    total_ms = 0.0
    for lg in range(1, 21):
        o2 = torch.from_numpy(inst.equal_offsets(n2, 1 << lg)).to(dev)
        t = _timed(stream, lambda: L.segsort_pairs_u32(kk.data_ptr(), vv.data_ptr(), n2,
                                                       o2.data_ptr(), o2.numel() - 1, st),
                   restore4, warmup, steps)
        ms = statistics.median(t)
        per[lg] = round(ms, 4)
        total_ms += ms
    out["pairs_2e24_keys_0_16_sweep"] = {
        "ms_per_len": per, "gkeys_s": round(20 * n2 / (total_ms * 1e-3) / 1e9, 3)}
    if pkg.device_status() != 0:
        raise RuntimeError("device status reports a bounded wait that gave up")
    return out


# ---------------------------------------------------------------------------
def run_ours(args) -> None:
    import torch
    import torch.distributed as dist

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)

    pkg = entry.load_package()
    pkg.build()
    inst = importlib.import_module(f"{entry.PKG_NAME}.instances")
    L = pkg.lib()
    lengths = log_lengths(args.lengths)
    n = 1 << args.log_n
    stream = torch.cuda.current_stream()
    st = stream.cuda_stream

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    # ---- inputs: one fresh copy per (step, length), all resident ----------
    offsets = {lg: torch.from_numpy(inst.equal_offsets(n, 1 << lg)).to(dev) for lg in lengths}
    pristine = {lg: inst.device_uniform_keys(n, seed=1000 + lg, bits=32, device=dev)
                for lg in lengths}
    ar = torch.arange(n, dtype=torch.int32, device=dev)
    total_steps = args.warmup + args.steps
    bufs = [{lg: (pristine[lg].clone(), ar.clone()) for lg in lengths} for _ in range(total_steps)]
    torch.cuda.synchronize()

    def sort_call(k, v, lg):
        o = offsets[lg]
        rc = L.segsort_pairs_u32(k.data_ptr(), v.data_ptr(), n, o.data_ptr(), o.numel() - 1, st)
        if rc != 0:
            raise pkg.SegsortError(rc, "segsort_pairs_u32")

    for s in range(args.warmup):
        for lg in lengths:
            sort_call(*bufs[s][lg], lg)
    barrier()
    if pkg.device_status() != 0:
        raise RuntimeError("device status reports a bounded wait that gave up")

    # ---- timed region: exactly K steps -------------------------------------
    evs = {lg: [] for lg in lengths}
    gpu_uuid = None
    try:
        gpu_uuid = str(torch.cuda.get_device_properties(dev).uuid)
        gpu_uuid = gpu_uuid if gpu_uuid.startswith("GPU-") else "GPU-" + gpu_uuid
    except Exception:
        gpu_uuid = None
    with ClockSampler(gpu_uuid) as clocks:
        barrier()
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        t_start.record(stream)
        for s in range(args.warmup, total_steps):
            for lg in lengths:
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                sort_call(*bufs[s][lg], lg)
                b.record(stream)
                evs[lg].append((a, b))
        t_end.record(stream)
        barrier()
    region_ms = max_over_ranks(t_start.elapsed_time(t_end), world, dev)
    keys_per_step = n * len(lengths)
    value = whole_job_gkeys(keys_per_step, args.steps, world, region_ms)
    if pkg.device_status() != 0:
        raise RuntimeError("device status reports a bounded wait that gave up")

    peak, peak_kind = peak_hbm()
    per_len = []
    for lg in lengths:
        ms = statistics.median(a.elapsed_time(b) for a, b in evs[lg])
        gbs = (BYTES_PER_PAIR * n + 4 * (n // (1 << lg) + 1)) / (ms * 1e-3) / 1e9
        per_len.append({"log2_len": lg, "ms": round(ms, 5),
                        "gkeys_s": round(n / (ms * 1e-3) / 1e9, 3),
                        "hbm_frac": round(gbs / peak, 4)})
    del bufs

    # ---- phase profile (one more step on fresh copies) ---------------------
    pkg.profile_enable(True)
    pkg.profile_read(reset=True)
    phase = {}
    for lg in lengths:
        k, v = pristine[lg].clone(), ar.clone()
        torch.cuda.synchronize()
        sort_call(k, v, lg)
        torch.cuda.synchronize()
        phase[lg] = pkg.profile_read(reset=True)
    pkg.profile_enable(False)
    cap = 4096  # tile capacity of 32-bit keys: longer segments take a long-segment route
    radix_min = pkg.get_param(pkg.PARAM_RADIX_MIN_32)
    stream_max_avg = pkg.get_param(pkg.PARAM_STREAM_MAX_AVG)
    bucket_min_avg = pkg.get_param(pkg.PARAM_BUCKET_MIN_AVG)
    msd_on = pkg.get_param(pkg.PARAM_MSD)
    tiny_max_avg = pkg.get_param(pkg.PARAM_TINY_MAX_AVG)
    launches_per_step = sum(p["tile_launches"] + p["large_launches"] for p in phase.values())

    def merge_passes(length: int) -> int:
        runs, p = -(-length // cap), 0
        while runs > 1:
            runs, p = (runs + 1) // 2, p + 1
        return p

    def varying_digits(lg: int) -> list[int]:
        """8-bit digit positions whose value differs somewhere inside a
        segment of the instance: the radix passes the library runs."""
        k = pristine[lg].long() & 0xFFFFFFFF
        seg = torch.arange(n, device=dev) >> lg
        out = []
        for d in range(4):
            dg = (k >> (8 * d)) & 255
            lo = torch.full((n >> lg,), 256, dtype=torch.long, device=dev).scatter_reduce(
                0, seg, dg, reduce="amin")
            hi = torch.full((n >> lg,), -1, dtype=torch.long, device=dev).scatter_reduce(
                0, seg, dg, reduce="amax")
            if bool((lo != hi).any()):
                out.append(d)
        return out

    def msd_oversize_bytes(lg: int, d: int) -> int:
        """Merge-pass bytes of the sub-buckets (segment, value of digit d)
        longer than a tile: the MSD route's second stage gives each of them
        merge_passes(length) passes (sub-buckets are at most four tiles)."""
        k = pristine[lg].long() & 0xFFFFFFFF
        sub = ((torch.arange(n, device=dev) >> lg) << 8) | ((k >> (8 * d)) & 255)
        c = torch.bincount(sub, minlength=(n >> lg) << 8)
        big = c[c > cap].tolist()
        return sum(BYTES_PER_PAIR * x * merge_passes(x) for x in big)

    # Algorithmic bytes per launch.  The tile kernels read and write every
    # key and value once and read the offsets: all of them when the segments
    # are at most a tile long, the long segments' elements when they form
    # their sorted runs for the merge passes.  A merge pass reads and writes
    # every key and value of its segments once.  The LSD radix route reads
    # every key once for the digit counts, then reads and writes every key and
    # value once per digit position that varies, plus one copy back after an
    # odd number of passes.  The MSD route (segments longer than the radix
    # threshold whose keys vary in at least three digits) reads every key for
    # the counts and every pair once in its one pass (long-segment kernel),
    # then every pair once in the bucket kernel, plus a merge pass over the
    # sub-buckets longer than a tile.  The library runs the tiny route
    # (tile_tiny_kernel, and tile_list_kernel for the chunks it lists) when
    # the average segment is at most tiny_max_avg long, the streamed tile
    # kernel when it is at most stream_max_avg long, the bucket route
    # (tile_bucket_kernel, and tile_list_kernel for the chunks it refuses)
    # from bucket_min_avg on, the one-CTA-per-tile comparison sort between.
    tile_bytes, stream_bytes, bucket_bytes, long_bytes, idle_tile = {}, {}, {}, {}, []
    tiny_bytes = {}
    route = {}  # per length, the route its call takes (reported with per_len)
    for lg in lengths:
        ln = 1 << lg
        full = BYTES_PER_PAIR * n + 4 * (n // ln + 1)
        bucket = bool(bucket_min_avg) and ln >= bucket_min_avg
        tile_table = bucket_bytes if bucket else tile_bytes
        if ln <= stream_max_avg and ln <= tiny_max_avg:
            tiny_bytes[lg] = full
            route[lg] = "tiny"
        elif ln <= stream_max_avg:
            stream_bytes[lg] = full
            route[lg] = "streamed tile"
        elif ln <= cap:
            tile_table[lg] = full
            route[lg] = "bucket" if bucket else "comparison tile"
        elif ln <= radix_min:
            tile_table[lg] = full
            long_bytes[lg] = BYTES_PER_PAIR * n * merge_passes(ln)
            route[lg] = f"{'bucket' if bucket else 'comparison'}-sorted runs + {merge_passes(ln)} merge passes"
        else:
            digits = varying_digits(lg)
            if msd_on and len(digits) >= 3:
                bucket_bytes[lg] = BYTES_PER_PAIR * n
                long_bytes[lg] = 4 * n + BYTES_PER_PAIR * n + msd_oversize_bytes(lg, digits[-1])
                route[lg] = "MSD radix pass + bucket sort of the sub-buckets"
            else:
                idle_tile.append(lg)  # the tile kernel finds no work: every segment is on the radix route
                passes = len(digits)
                long_bytes[lg] = 4 * n + BYTES_PER_PAIR * n * (passes + (passes & 1))
                route[lg] = f"LSD radix, {passes} passes"
    for p in per_len:
        p["route"] = route[p["log2_len"]]
    kernels = {}
    for name, table, key in (("tile_sort_kernel", tile_bytes, "tile_ms"),
                             ("tile_tiny_kernel", tiny_bytes, "tile_ms"),
                             ("tile_stream_kernel", stream_bytes, "tile_ms"),
                             ("tile_bucket_kernel", bucket_bytes, "tile_ms"),
                             ("long_segment_kernel", long_bytes, "large_ms")):
        ms_sum = sum(phase[lg][key] for lg in table)
        byts = sum(table.values())
        if ms_sum > 0 and table:
            kernels[name] = {"ms_per_step": round(ms_sum, 4), "launches_per_step": len(table),
                             "algorithmic_bytes_per_step": byts,
                             "achieved_gbs": round(byts / (ms_sum * 1e-3) / 1e9, 1)}
    if idle_tile:
        kernels["tile_sort_kernel_no_work"] = {
            "ms_per_step": round(sum(phase[lg]["tile_ms"] for lg in idle_tile), 4),
            "launches_per_step": len(idle_tile), "algorithmic_bytes_per_step": 0}
    name = max((k for k in kernels if kernels[k].get("algorithmic_bytes_per_step")),
               key=lambda k: kernels[k]["ms_per_step"])
    K = kernels[name]
    achieved = K["achieved_gbs"]
    tr = traffic_per_launch()
    roofline = {"bound": "hbm", "kernel": name, "achieved": achieved,
                "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                "peak_kind": f"{peak_kind} hbm_gbs (copy)",
                "algorithmic_bytes_per_launch": K["algorithmic_bytes_per_step"] // K["launches_per_step"],
                "traffic": ((tr or {}).get(name) or {}).get("dram_bytes_per_launch"),
                "traffic_workload": ((tr or {}).get(name) or {}).get("workload"),
                "radix_min": radix_min, "stream_max_avg": stream_max_avg,
                "bucket_min_avg": bucket_min_avg, "msd": msd_on,
                "tiny_max_avg": tiny_max_avg, "kernels": kernels}

    # ---- end to end through the public API with host buffers ---------------
    e2e = None
    if not args.no_e2e:
        host = {}
        for lg in lengths:
            hk = torch.empty(n, dtype=torch.int32, pin_memory=True)
            hk.copy_(pristine[lg].cpu())
            hv = torch.arange(n, dtype=torch.int32).pin_memory()
            host[lg] = (hk, hv, torch.empty(n, dtype=torch.int32, pin_memory=True),
                        torch.empty(n, dtype=torch.int32, pin_memory=True))
        # Four device slots on four streams: an instance's host-to-device copy,
        # the sorts and the device-to-host copies of earlier instances run at
        # once (both copy directions and the SMs).  Measured on GB300 with
        # 2^24 pairs per instance: four slots keep both link directions busy
        # (~95% of the concurrent copy limit), two leave them idle ~20% of the time.
        slots = [(torch.empty(n, dtype=torch.int32, device=dev),
                  torch.empty(n, dtype=torch.int32, device=dev),
                  torch.cuda.Stream(device=dev)) for _ in range(4)]

        def e2e_step():
            for i, lg in enumerate(lengths):
                hk, hv, ok, ov = host[lg]
                dk, dv, s = slots[i % len(slots)]
                with torch.cuda.stream(s):
                    dk.copy_(hk, non_blocking=True)
                    dv.copy_(hv, non_blocking=True)
                    pkg.segsort(dk, offsets[lg], dv, key_type="u32", stream=s)
                    ok.copy_(dk, non_blocking=True)
                    ov.copy_(dv, non_blocking=True)

        def join():
            for _, _, s in slots:
                stream.wait_stream(s)

        for _ in range(args.warmup):
            e2e_step()
        join()
        e_steps = max(1, min(args.steps, 5))
        barrier()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _, _, s in slots:
            s.wait_stream(stream)
        for _ in range(e_steps):
            e2e_step()
        join()
        b.record(stream)
        barrier()
        e_ms = max_over_ranks(a.elapsed_time(b), world, dev)
        e2e = {"value": whole_job_gkeys(keys_per_step, e_steps, world, e_ms), "unit": "Gkeys/s",
               "h2d_bytes_per_step": 8 * n * len(lengths),
               "d2h_bytes_per_step": 8 * n * len(lengths),
               "steps": e_steps, "ms_per_step": e_ms / e_steps}
        # Every instance read back into host memory holds its stable sort:
        # within each segment the values are a permutation of the segment's
        # positions, the keys moved with them, in order, ties in input order.
        for lg in lengths:
            hk, hv, ok, ov = host[lg]
            k = ok.to(dev).long() & 0xFFFFFFFF
            v = ov.to(dev).long() & 0xFFFFFFFF
            src = hk.to(dev).long() & 0xFFFFFFFF
            pos = torch.arange(n, device=dev)
            same = (pos[1:] >> lg) == (pos[:-1] >> lg)
            ok_all = (bool(((v >> lg) == (pos >> lg)).all())
                      and bool((torch.bincount(v, minlength=n) == 1).all())
                      and torch.equal(src[v], k)
                      and bool(((k[1:] > k[:-1]) | ~same | ((k[1:] == k[:-1]) & (v[1:] > v[:-1]))).all()))
            if not ok_all:
                raise RuntimeError(f"end-to-end read-back of segment length 2^{lg} is not its stable sort")
        e2e["checked"] = f"every instance read back ({len(lengths)} x {n} pairs)"

    # ---- the batched form and the other workloads ---------------------------
    batched = None if args.no_batched else bench_batched(pkg, inst, dev, stream, 2, 5)
    configs = None if args.no_configs else bench_configs(pkg, inst, dev, stream, 3, 10)
    served = None
    if rank == 0 and not args.no_served:
        served = bench_served(args.served_requests, args.served_rates)

    # ---- CPU baseline (rank 0): the same full instances, all host threads and
    # one thread -------------------------------------------------------------
    cpu = None
    if rank == 0 and not args.no_cpu:
        from oracle import oracle as O
        O.build()
        threads = O.default_threads()
        sweep = CpuSweep(O, inst, n, lengths)
        secs = sweep.step(threads)
        secs1 = sweep.step(1)
        cpu = {"value": sweep.keys_per_step / secs / 1e9, "unit": "Gkeys/s", "cores": threads,
               "kind": "port", "cpu_model": cpu_model(),
               "sample": f"one step of the full sweep ({len(lengths)} instances of {n} pairs), "
                         f"std::stable_sort per segment on {threads} threads",
               "single_thread": {"value": sweep.keys_per_step / secs1 / 1e9, "unit": "Gkeys/s",
                                 "cores": 1, "sample": "one step of the full sweep on 1 thread "
                                                      "(the reference's mseq is sequential)"}}
        del sweep

    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": "Gkeys/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": region_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": bench_config(n, lengths, world),
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": launches_per_step * args.steps,
            "clocks": clocks.summary(), "per_len": per_len,
            "batched": batched, "configs": configs, "served": served,
        }), flush=True)
    if world > 1:
        dist.destroy_process_group()


def run_served_only(args) -> None:
    entry.load_package().build()
    print(json.dumps({"metric": "served-form request stream (p50/p99/p999 ms, Gkeys/s)",
                      "served": bench_served(args.served_requests, args.served_rates)}), flush=True)


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.served_only:
        run_served_only(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
