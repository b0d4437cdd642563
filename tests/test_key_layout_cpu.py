"""The boundary key layouts of the device header, checked on the host: the
header's pack/unpack/row_successor are __host__ __device__, so a host-only
program compiled with nvcc runs them here without a GPU.

Every reachable boundary state of random placements round-trips through a
u64 key (the reference PackedBoundary layout, src/lib.rs:348-377, for N <= 21;
the compact 3N - 2-bit layout at N = 22) and through a u128 key; the u64 key
equals the reference layout bit for bit up to N = 21 and the u128 key's
reference layout at N = 22 with the two always-clear bits dropped; no u64 key
is all ones (the partitioned merge's empty-slot marker).
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

from conftest import ROOT

PROGRAM = r"""
#include <cstdio>
#include <random>
#include "qpeps_device.cuh"
using namespace qpeps;
int main() {
  std::mt19937_64 rng(20261204);
  long checked = 0;
  for (unsigned n : {1u, 2u, 8u, 13u, 16u, 20u, 21u, 22u}) {
    const u64 mask = (n >= 64) ? ~0ull : ((1ull << n) - 1);
    for (int trial = 0; trial < 4000; ++trial) {
      State s{0, 0, 0};
      for (unsigned row = 0; row < n; ++row) {
        const u64 fr = ~(s.cols | s.dr | s.dl) & mask;
        if (!fr) break;
        int k = (int)(rng() % (u64)__builtin_popcountll(fr));
        u64 f = fr;
        while (k--) f &= f - 1;
        const u64 b = f & (0ull - f);
        const u64 k64 = row_successor<u64>(s, b, n, mask);
        const u128 k128 = row_successor<u128>(s, b, n, mask);
        const State a = unpack<u64>(k64, n, mask), c = unpack<u128>(k128, n, mask);
        if (a.cols != c.cols || a.dr != c.dr || a.dl != c.dl) { std::printf("FAIL roundtrip n=%u\n", n); return 1; }
        if (pack<u64>(a.cols, a.dr, a.dl, n) != k64) { std::printf("FAIL repack n=%u\n", n); return 1; }
        if (k64 == ~0ull) { std::printf("FAIL empty marker n=%u\n", n); return 1; }
        const u128 ref = (u128)a.cols | ((u128)a.dr << n) | ((u128)a.dl << (2 * n));
        if (k128 != ref) { std::printf("FAIL u128 layout n=%u\n", n); return 1; }
        if (n <= 21 && (u128)k64 != ref) { std::printf("FAIL u64 reference layout n=%u\n", n); return 1; }
        if (n == 22 && ((a.dr & 1ull) || (a.dl >> 21))) { std::printf("FAIL live bits n=%u\n", n); return 1; }
        if (n == 22 && k64 != (u64)(a.cols | ((a.dr >> 1) << 22) | (a.dl << 43))) {
          std::printf("FAIL compact layout n=%u\n", n); return 1;
        }
        s = a;
        ++checked;
      }
    }
  }
  std::printf("OK %ld\n", checked);
  return 0;
}
"""


def test_key_layouts_round_trip_on_the_host(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    src = tmp_path / "layout.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "layout"
    csrc = ROOT / "quantum-harness-peps-naive_gb300" / "csrc"
    build = subprocess.run([nvcc, "-O2", "-std=c++17", "-I", str(csrc), str(src), "-o", str(exe)],
                           capture_output=True, text=True, timeout=300)
    assert build.returncode == 0, build.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stdout + run.stderr
    assert run.stdout.startswith("OK ") and int(run.stdout.split()[1]) > 100000
