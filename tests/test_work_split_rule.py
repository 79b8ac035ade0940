"""The rule that cuts the edge phase's work into item ranges (work_parts in
csrc/acg_internal.h), compiled on the host: one range per launched warp for a
static split or little work, otherwise ranges of at least kMinRangeSteps load
steps each, at most max_ranges per warp -- and always a whole number of ranges
per warp, so that every launched warp owns a first range."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
CSRC = ROOT / "application_classification_gb300" / "csrc"

PROBE = r"""
#include <cstdio>
#include "acg_internal.h"
int main() {
  // up to totals past 2^32 steps (graphs of hundreds of millions of vertices)
  const double totals[] = {0, 1, 100, 15000, 77824, 1e6, 1.2e7, 1e9, 3e9, 6e10};
  const int warps[] = {1, 1216, 4864};
  const int maxr[] = {1, 16, 32};
  for (double t : totals)
    for (int w : warps)
      for (int m : maxr) std::printf("%.0f %d %d %d\n", t, w, m, acg::work_parts(t, w, m));
  std::printf("min %d\n", acg::kMinRangeSteps);
  return 0;
}
"""


def _cuda_include():
    for p in ("/usr/local/cuda/include", "/usr/local/cuda/targets/x86_64-linux/include"):
        if (Path(p) / "cuda_runtime.h").exists():
            return p
    return None


def test_work_parts_rule(tmp_path):
    cxx = shutil.which("g++")
    inc = _cuda_include()
    if not cxx or not inc:
        pytest.skip("needs g++ and the CUDA headers")
    src = tmp_path / "probe.cpp"
    src.write_text(PROBE)
    exe = tmp_path / "probe"
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", str(ROOT / "include"), "-I", str(CSRC),
                    "-I", inc, str(src), "-o", str(exe)], check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    kmin = int(out[-2].split()[1])
    for line in out[:-2]:
        t, w, m, parts = (float(x) for x in line.split())
        w, m, parts = int(w), int(m), int(parts)
        assert parts % w == 0 and parts >= w  # every launched warp owns a first range
        r = parts // w
        if m <= 1:
            assert r == 1  # a static split
        else:
            assert 1 <= r <= m
            # ranges of at least kMinRangeSteps steps, as many as that allows
            assert r == max(1, min(m, int(t / w / kmin)))
