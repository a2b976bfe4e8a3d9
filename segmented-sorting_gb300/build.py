"""Build recipe of the GB300 segmented sort (in-tree, no cmake).

Products, all written next to this file:
  libsegsort.so          the C-ABI library (csrc/segsort_api.cu: plain calls,
                         csrc/segsort_batch.cu: batched form,
                         csrc/segsort_server.cu: served form,
                         csrc/segsort_ext.cu: descending, top-k, 64-bit
                         values; sm_103a)
  serve_bench.exe        served-form benchmark driver (Poisson request stream)
  segsort_driver.exe     reference-compatible bench driver, prints sorted keys
  segsort_driver_time.exe  the same driver built with ELAPSED_TIME=1
                           EXECUTIONS=10: prints one ms line per execution
  gen_instance.exe       seeded instance generator (reference text format)

Every step runs only when an input is newer than its output.  Steps run in
parallel; the whole build takes well under a minute.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
REPO = PKG.parent
INCLUDE = REPO / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]

LIB = PKG / "libsegsort.so"
DRIVER = PKG / "segsort_driver.exe"
DRIVER_TIME = PKG / "segsort_driver_time.exe"
GEN = PKG / "gen_instance.exe"
SERVE = PKG / "serve_bench.exe"


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return p


def cuda_home() -> Path:
    return Path(nvcc()).resolve().parent.parent


def _stale(out: Path, inputs: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(p.stat().st_mtime > t for p in inputs)


def _run(cmd: list[str], verbose: bool) -> None:
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


OBJ_DIR = PKG / "_build"
LIB_UNITS = ["segsort_api.cu", "segsort_batch.cu", "segsort_server.cu", "segsort_ext.cu"]


def _obj(unit: str) -> Path:
    return OBJ_DIR / (Path(unit).stem + ".o")


def _obj_cmd(unit: str) -> list[str]:
    return [nvcc(), *ARCH, *NVCC_FLAGS, f"-I{INCLUDE}", "-c", str(CSRC / unit), "-o", str(_obj(unit))]


def _lib_cmd() -> list[str]:
    return [nvcc(), *ARCH, "-shared", *[str(_obj(u)) for u in LIB_UNITS], "-o", str(LIB)]


def _driver_cmd(out: Path, timed: bool) -> list[str]:
    cuda = cuda_home()
    defs = ["-DELAPSED_TIME=1", "-DEXECUTIONS=10"] if timed else ["-DELAPSED_TIME=0", "-DEXECUTIONS=1"]
    return ["g++", "-O2", "-std=c++17", *defs, f"-I{INCLUDE}", f"-I{cuda / 'include'}",
            str(CSRC / "segsort_driver.cpp"), "-o", str(out), f"-L{PKG}", "-lsegsort",
            f"-L{cuda / 'lib64'}", "-lcudart", "-Wl,-rpath,$ORIGIN",
            f"-Wl,-rpath,{cuda / 'lib64'}"]


def _serve_cmd() -> list[str]:
    cuda = cuda_home()
    return ["g++", "-O2", "-std=c++17", "-pthread", f"-I{INCLUDE}", f"-I{cuda / 'include'}",
            str(CSRC / "serve_bench.cpp"), "-o", str(SERVE), f"-L{PKG}", "-lsegsort",
            f"-L{cuda / 'lib64'}", "-lcudart", "-Wl,-rpath,$ORIGIN", f"-Wl,-rpath,{cuda / 'lib64'}"]


def _gen_cmd() -> list[str]:
    return ["g++", "-O2", "-std=c++17", str(CSRC / "gen_instance.cpp"), "-o", str(GEN)]


def lib_sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cuh")) + [INCLUDE / "segsort.h"]


def build(verbose: bool = False) -> None:
    """Compile the library, the drivers and the generator for sm_103a."""
    lib_in = lib_sources()
    OBJ_DIR.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.cuh")) + [INCLUDE / "segsort.h"]
    units = [u for u in LIB_UNITS if _stale(_obj(u), [CSRC / u, *headers])]
    with ThreadPoolExecutor(max_workers=max(1, len(units))) as ex:
        for f in [ex.submit(_run, _obj_cmd(u), verbose) for u in units]:
            f.result()
    if _stale(LIB, [_obj(u) for u in LIB_UNITS]):
        _run(_lib_cmd(), verbose)
    jobs = []
    drv_in = [CSRC / "segsort_driver.cpp", INCLUDE / "segsort.h", LIB]
    if _stale(DRIVER, drv_in):
        jobs.append(_driver_cmd(DRIVER, False))
    if _stale(DRIVER_TIME, drv_in):
        jobs.append(_driver_cmd(DRIVER_TIME, True))
    if _stale(GEN, [CSRC / "gen_instance.cpp"]):
        jobs.append(_gen_cmd())
    if _stale(SERVE, [CSRC / "serve_bench.cpp", INCLUDE / "segsort.h", LIB]):
        jobs.append(_serve_cmd())
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for f in [ex.submit(_run, j, verbose) for j in jobs]:
            f.result()


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
