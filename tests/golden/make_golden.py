"""Regenerate the golden fixtures in this directory from the reference itself.

Each fixture <name>.npz holds one instance and the reference's own answers:
  offsets, keys            the instance (CSR offsets, uint32 keys)
  ref_keys                 stdout of the reference's CPU sort mseq
                           (src/mseq.cu, per-segment std::stable_sort of keys)
  ref_pair_keys, ref_pair_vals
                           the reference's pair oracle gold_segsort
                           (src/bb_segsort/main.cu:152-173) on (key, index)
Both programs are built from the reference sources by `make -C oracle ref`
(outputs in the git-ignored oracle/_ref/).  Running this script needs the
reference checkout; the committed .npz files do not.

Instances: the reference's two shipped inputs (src/mergesort2/in1-32 and
in2-1024, read at generation time) and seeded instances from
segmented-sorting_gb300/instances.py covering equal, random-cut (gen_diff),
lognormal-with-empty-segments and low-entropy keys, segment lengths around
the tile capacity (4096) and the reference's bin edges, and the largest key
the reference's "%d" reader accepts (2^31 - 1).
"""
from __future__ import annotations

import importlib.util
import subprocess
import sys
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
REF = Path(os.environ.get("SEGSORT_REF_DIR", "/root/reference"))
sys.path.insert(0, str(REPO))

from oracle import oracle as O  # noqa: E402

spec = importlib.util.spec_from_file_location(
    "segsort_instances", REPO / "segmented-sorting_gb300" / "instances.py")
inst = importlib.util.module_from_spec(spec)
spec.loader.exec_module(inst)


def parse_c1(text: str):
    tok = text.split()
    nseg = int(tok[0])
    off = np.array(tok[1:nseg + 2], dtype=np.int64)
    n = int(tok[nseg + 2])
    keys = np.array(tok[nseg + 3:nseg + 3 + n], dtype=np.int64)
    return off.astype(np.int32), keys.astype(np.uint32)


def run_gold(off: np.ndarray, keys: np.ndarray):
    out = subprocess.run([str(O.HERE / "_ref" / "gold_segsort.exe")], input=O.c1_text(off, keys),
                         text=True, capture_output=True, check=True).stdout.split("\n")
    k = np.array(out[0].split(), dtype=np.int64).astype(np.uint32)
    v = np.array(out[1].split(), dtype=np.int64).astype(np.uint32)
    return k, v


def cases():
    for name in ("in1-32", "in2-1024"):
        p = REF / "src" / "mergesort2" / name
        yield f"ref_{name.replace('-', '_')}", *parse_c1(p.read_text())
    yield "equal_len2_bits12", inst.equal_offsets(8192, 2), inst.uniform_keys(8192, 11, 12)
    yield "equal_len32_bits12", inst.equal_offsets(8192, 32), inst.uniform_keys(8192, 12, 12)
    yield "equal_len1024_bits31", inst.equal_offsets(8192, 1024), inst.uniform_keys(8192, 13, 31)
    yield "equal_len256_bits4", inst.equal_offsets(8192, 256), inst.uniform_keys(8192, 14, 4)
    yield "single_4096_bits31", np.array([0, 4096], np.int32), inst.uniform_keys(4096, 15, 31)
    yield "single_4097_bits31", np.array([0, 4097], np.int32), inst.uniform_keys(4097, 16, 31)
    yield "single_9000_bits8", np.array([0, 9000], np.int32), inst.uniform_keys(9000, 17, 8)
    yield "diff_37_bits12", inst.diff_offsets(10000, 37, 18), inst.uniform_keys(10000, 18, 12)
    yield "diff_3_bits31", inst.diff_offsets(15000, 3, 19), inst.uniform_keys(15000, 19, 31)
    yield "lognormal_bits31", inst.lognormal_offsets(12000, 20, empty_frac=0.05), \
        inst.uniform_keys(12000, 20, 31)
    # Lengths at the reference's bin edges (src/bb_segsort/bb_bin.h:67-91) and
    # around the tile capacity, with empty segments in between.
    lens = [0, 1, 2, 3, 4, 5, 8, 9, 16, 17, 32, 33, 64, 65, 128, 129, 256, 257, 0, 512, 513,
            1024, 1025, 2048, 2049, 0, 0, 4095, 4096, 4097, 1]
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    k = inst.uniform_keys(int(off[-1]), 21, 31)
    k[::7] = 2**31 - 1  # the largest key the reference reads with "%d"
    yield "bin_edges_maxkey", off, k


def main() -> None:
    subprocess.run(["make", "-s", "-C", str(O.HERE), "all", "ref"], check=True)
    for name, off, keys in cases():
        ref_keys = O.run_reference_mseq(off, keys)
        pk, pv = run_gold(off, keys)
        np.savez_compressed(HERE / f"{name}.npz", offsets=off, keys=keys, ref_keys=ref_keys,
                            ref_pair_keys=pk, ref_pair_vals=pv)
        print(f"{name}: nseg={len(off) - 1} n={len(keys)}")


if __name__ == "__main__":
    main()
