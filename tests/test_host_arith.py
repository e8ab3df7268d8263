"""Host-side integer arithmetic of the CUDA library, run on the CPU: the
multiply-shift division (FastDiv in csrc/common.cuh) that the mixed-path
kernels use to split extended neighbour indices e = s * nloc + j and row
indices, against exact integer division over divisors 1 .. 5000, powers of
two and their neighbours, and random 31-bit divisors, each with edge and
random numerators.  The header is compiled into a small host program with
nvcc (its __host__ __device__ member runs on the CPU)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)

PROGRAM = r"""
#include <cstdio>
#include "common.cuh"
int main() {
  int d, n;
  while (std::scanf("%d %d", &d, &n) == 2) std::printf("%d\n", dpgb::FastDiv(d).div(n));
  return 0;
}
"""


def _cases():
    rng = np.random.default_rng(11)
    ds = list(range(1, 5001))
    for l in range(1, 31):
        ds += [(1 << l) - 1, 1 << l, (1 << l) + 1]
    ds += [int(x) for x in rng.integers(1, 2**31 - 1, size=2000)]
    out = []
    top = 2**31 - 1
    for d in ds:
        d = min(d, top)
        ns = {0, 1, d - 1, d, d + 1, top, top - 1, top // d * d, max(top // d * d - 1, 0)}
        ns |= {int(x) for x in rng.integers(0, top, size=3)}
        out += [(d, n) for n in sorted(ns) if 0 <= n <= top]
    return out


def test_fastdiv_matches_integer_division(tmp_path):
    nvcc = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)
    if nvcc is None:
        pytest.skip("nvcc not available")
    src = tmp_path / "fastdiv.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "fastdiv"
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-I", os.path.join(REPO, "include"), "-I",
                        os.path.join(REPO, "deepmd-kit_gb300", "csrc"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    cases = _cases()
    feed = "\n".join(f"{d} {n}" for d, n in cases) + "\n"
    r = subprocess.run([str(exe)], input=feed, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = [int(x) for x in r.stdout.split()]
    want = [n // d for d, n in cases]
    assert len(got) == len(want)
    bad = [(d, n, g, w) for (d, n), g, w in zip(cases, got, want) if g != w]
    assert not bad, bad[:10]
