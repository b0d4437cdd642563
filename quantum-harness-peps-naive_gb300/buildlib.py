"""Build the CUDA library in-tree: libqpeps.so (sm_103a) and the qpeps CLI.

    python quantum-harness-peps-naive_gb300/buildlib.py

Translation units are compiled in parallel with nvcc and linked into
`libqpeps.so` next to this file (git-ignored). The CLI links against it with an
$ORIGIN rpath.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIB = PKG / "libqpeps.so"
CLI = PKG / "qpeps"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-Xcompiler",
    "-fPIC",
    "--expt-relaxed-constexpr",
    "-I",
    str(INCLUDE),
]
LIB_SOURCES = ["qpeps_hash_kernels.cu", "qpeps_partition_kernels.cu", "qpeps_unit_kernels.cu", "qpeps_wide_kernels.cu",
               "qpeps_engine.cu", "qpeps_noalloc.cu", "qpeps_tail_kernels.cu", "qpeps_probe_kernels.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False) -> Path:
    OBJ.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [INCLUDE / "qpeps.h"]
    nv = nvcc()
    jobs = []
    objs = []
    for src in LIB_SOURCES:
        s = CSRC / src
        o = OBJ / (s.stem + ".o")
        objs.append(o)
        if _stale(o, [s] + headers):
            jobs.append([nv, *NVCC_FLAGS, "-c", str(s), "-o", str(o)])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            for f in [ex.submit(_run, j) for j in jobs]:
                f.result()
    if jobs or _stale(LIB, objs):
        _run([nv, *ARCH, "-shared", "-o", str(LIB), *map(str, objs)])
    cli_src = CSRC / "qpeps_cli.cpp"
    if cli_src.exists() and _stale(CLI, [cli_src, LIB, INCLUDE / "qpeps.h"]):
        _run(
            [
                "g++",
                "-O2",
                "-std=c++17",
                "-I",
                str(INCLUDE),
                str(cli_src),
                "-L",
                str(PKG),
                "-lqpeps",
                "-Wl,-rpath,$ORIGIN",
                "-o",
                str(CLI),
            ]
        )
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
