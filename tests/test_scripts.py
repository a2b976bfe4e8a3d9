"""The reference's benchmark scripts run unchanged against this build's driver.

The reference times each variant with a loop (scripts/exec.sh:5-21) that
walks a directory of instances named <nseg>_<n>.in in creation order
(`ls -tr`), prints a blank line, nseg and n before each instance, and feeds
the instance to the program on stdin; the program prints one ms line per
execution (src/mseq.cu:84-89, EXECUTIONS = 10).  utils/parser.cpp:22-83 then
reads that output back: a header line, then per size n a run of blocks
(nseg, n, ten times) that ends at the block with nseg >= n / 2.

Here segsort_driver_time.exe (ELAPSED_TIME = 1, EXECUTIONS = 10) stands in
for the reference's program.  The instances are written by gen_instance.exe
in the order scripts/genequalseg.sh creates them (for each n, nseg = 1, 2, 4,
... below n), and the loop and the parser's rules are restated below.  Where
the reference checkout is mounted (SEGSORT_REF_DIR, default /root/reference)
its own exec.sh runs too and must print the same structure.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

import pytest

SIZES = (1024, 4096)
EXECUTIONS = 10


def _make_instances(pkg, d: Path) -> list[Path]:
    """<nseg>_<n>.in for every n in SIZES and nseg = 1, 2, ... < n, with
    increasing modification times (the order `ls -tr` lists them in)."""
    gen = pkg.PKG / "gen_instance.exe"
    files, stamp = [], 1_600_000_000
    for n in SIZES:
        nseg = 1
        while nseg < n:
            f = d / f"{nseg}_{n}.in"
            data = subprocess.run([str(gen), "equal", str(nseg), str(n // nseg), "--bits", "12"],
                                  capture_output=True, check=True).stdout
            f.write_bytes(data)
            os.utime(f, (stamp, stamp))
            stamp += 1
            files.append(f)
            nseg *= 2
    return files


def _exec_loop(prog: Path, d: Path) -> str:
    """scripts/exec.sh restated: instances in modification-time order; a
    blank line, nseg and n whenever nseg changes; the program on stdin."""
    out, c_aux = [], None
    for f in sorted(d.iterdir(), key=lambda p: p.stat().st_mtime):
        c, n = f.stem.split("_")[:2]
        if c != c_aux:
            out += [" ", c, n]
            c_aux = c
        with open(f, "rb") as fh:
            r = subprocess.run([str(prog)], stdin=fh, capture_output=True, text=True, check=True)
        out.append(r.stdout.rstrip("\n"))
    return "\n".join(out) + "\n"


def _parse(text: str, segments_cap: int = 8388608) -> list[list[tuple[int, list[float]]]]:
    """utils/parser.cpp's reading rules: a header line; per size a run of
    blocks (nseg line, n line, EXECUTIONS time lines, a separator line),
    closed by the block whose nseg reaches n / 2 (or the cap)."""
    lines = text.split("\n")
    pos = 1  # the header line
    sizes = []
    while pos < len(lines) and lines[pos].strip():
        seg = int(lines[pos]); size = int(lines[pos + 1]); pos += 2
        blocks = []
        while True:
            times = [float(x) for x in lines[pos:pos + EXECUTIONS]]
            assert len(times) == EXECUTIONS
            pos += EXECUTIONS
            blocks.append((size, seg, times))
            pos += 1  # separator
            if seg >= segments_cap or seg >= size // 2:
                break
            seg = int(lines[pos]); size = int(lines[pos + 1]); pos += 2
        sizes.append(blocks)
    return sizes


def _check(parsed):
    assert [blocks[0][0] for blocks in parsed] == list(SIZES)
    for blocks, n in zip(parsed, SIZES):
        assert [b[1] for b in blocks] == [1 << i for i in range(n.bit_length() - 1)]
        for _, _, times in blocks:
            assert all(t > 0.0 for t in times)


@pytest.mark.gpu
def test_exec_loop_and_parser_rules(pkg, cuda, tmp_path):
    d = tmp_path / "inst"
    d.mkdir()
    _make_instances(pkg, d)
    text = _exec_loop(pkg.PKG / "segsort_driver_time.exe", d)
    _check(_parse(text))


@pytest.mark.gpu
def test_reference_exec_script_when_mounted(pkg, cuda, tmp_path):
    ref = Path(os.environ.get("SEGSORT_REF_DIR", "/root/reference"))
    script = ref / "scripts" / "exec.sh"
    if not script.exists():
        pytest.skip("reference checkout not mounted")
    d = tmp_path / "inst"
    d.mkdir()
    _make_instances(pkg, d)
    work = tmp_path / "run"
    work.mkdir()
    (work / "prog").symlink_to(pkg.PKG / "segsort_driver_time.exe")
    r = subprocess.run(["bash", str(script), "prog", str(d)], cwd=work, capture_output=True,
                       text=True, check=True)
    _check(_parse(r.stdout))


def test_restated_loop_matches_the_reference_script(pkg, tmp_path):
    """CPU: where the reference checkout is mounted, its exec.sh and the
    restated loop print the same bytes over the same instances, with a
    stand-in program that prints ten times; the parser rules accept it."""
    ref = Path(os.environ.get("SEGSORT_REF_DIR", "/root/reference"))
    script = ref / "scripts" / "exec.sh"
    if not script.exists():
        pytest.skip("reference checkout not mounted")
    d = tmp_path / "inst"
    d.mkdir()
    _make_instances(pkg, d)
    work = tmp_path / "run"
    work.mkdir()
    prog = work / "prog"
    prog.write_text("#!/bin/bash\ncat > /dev/null\nfor i in 1 2 3 4 5 6 7 8 9 10; do echo 0.25$i; done\n")
    prog.chmod(0o755)
    r = subprocess.run(["bash", str(script), "prog", str(d)], cwd=work, capture_output=True,
                       text=True, check=True)
    assert r.stdout == _exec_loop(prog, d)
    _check(_parse(r.stdout))
