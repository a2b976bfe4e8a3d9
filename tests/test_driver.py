"""The reference-compatible command-line programs: gen_instance.exe writes the
reference's instance text (utils/gen_equal.cpp:108-114) and the binary
instance format; segsort_driver.exe reads either from stdin and prints the
sorted keys like src/mseq.cu:27-33 or one ms line per execution like
src/mseq.cu:84-89.  CPU tests check the generator against the Python
generator and the two formats against each other; GPU tests run the driver."""
from __future__ import annotations

import subprocess

import numpy as np
import pytest


def _gen(pkg, *args) -> bytes:
    exe = pkg.PKG / "gen_instance.exe"
    return subprocess.run([str(exe), *args], capture_output=True, check=True).stdout


def _parse_text(data: bytes):
    tok = data.split()
    nseg = int(tok[0])
    off = np.array([int(x) for x in tok[1:nseg + 2]], dtype=np.int64)
    n = int(tok[nseg + 2])
    keys = np.array([int(x) for x in tok[nseg + 3:nseg + 3 + n]], dtype=np.uint64)
    return off, keys


@pytest.mark.parametrize("args", [["equal", "8", "100"], ["diff", "9", "1000"],
                                  ["lognormal", "5000"]])
def test_generator_text_and_binary_agree(pkg, inst, args):
    for bits in ("12", "32"):
        text = _gen(pkg, *args, "--bits", bits, "--seed", "5")
        binary = _gen(pkg, *args, "--bits", bits, "--seed", "5", "--binary")
        off_t, keys_t = _parse_text(text)
        off_b, keys_b = inst.read_binary_instance(binary)
        assert np.array_equal(off_t, off_b.astype(np.int64))
        assert keys_b.dtype == np.uint32 and np.array_equal(keys_t, keys_b.astype(np.uint64))
        # keys are the counter-based stream of instances.py
        assert np.array_equal(keys_b, inst.uniform_keys(len(keys_b), 5, int(bits)))


def test_binary_writer_round_trip(inst):
    rng = np.random.default_rng(1)
    for dt in (np.uint32, np.int32, np.float32, np.uint64):
        keys = rng.integers(0, 1000, 77).astype(dt)
        off = np.array([0, 3, 3, 50, 77], np.int32)
        o, k = inst.read_binary_instance(inst.write_binary_instance(off, keys))
        assert np.array_equal(o, off) and k.dtype == dt and np.array_equal(k, keys)


def _drive(pkg, data: bytes, *opts, via_file=None) -> bytes:
    exe = pkg.PKG / "segsort_driver.exe"
    if via_file is not None:
        via_file.write_bytes(data)
        with open(via_file, "rb") as f:
            return subprocess.run([str(exe), *opts], stdin=f, capture_output=True, check=True).stdout
    return subprocess.run([str(exe), *opts], input=data, capture_output=True, check=True).stdout


@pytest.mark.gpu
def test_driver_prints_sorted_keys_for_text_and_binary(pkg, inst, oracle, tmp_path, cuda):
    text = _gen(pkg, "lognormal", "30000", "--bits", "32", "--seed", "9")
    binary = _gen(pkg, "lognormal", "30000", "--bits", "32", "--seed", "9", "--binary")
    off, keys = inst.read_binary_instance(binary)
    expect = oracle.segsort_numpy(keys, off)
    out_text = _drive(pkg, text, "--print")
    out_pipe = _drive(pkg, binary, "--print")
    out_mmap = _drive(pkg, binary, "--print", via_file=tmp_path / "inst.bin")
    got = np.array([int(x) for x in out_text.split()], dtype=np.uint64)
    assert np.array_equal(got, expect.astype(np.uint64))
    assert out_text == out_pipe == out_mmap
    # pairs: values are input positions, printed after the keys
    out_pairs = _drive(pkg, binary, "--print", "--pairs", "--print-values")
    lines = out_pairs.split(b"\n")
    vals = np.array([int(x) for x in lines[2].split()], dtype=np.uint32)
    ek, ev = oracle.segsort_numpy(keys, off, np.arange(len(keys), dtype=np.uint32))
    assert np.array_equal(vals, ev)


@pytest.mark.gpu
def test_driver_timing_lines(pkg, cuda):
    data = _gen(pkg, "equal", "64", "4096", "--bits", "32")
    out = _drive(pkg, data, "--time", "--execs", "3")
    ms = [float(x) for x in out.split()]
    assert len(ms) == 3 and all(t > 0 for t in ms)
