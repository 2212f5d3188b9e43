"""The tiled push's cell windows: the consumer warps find a cell's row with
window_slot and the producer warp stages segment s's rows from
segment_start, so the two must describe the same map.  The functions of
push_impl.cuh are compiled for the host (nvcc, no GPU) with each window shape
(CPIC_TILE_WINDOW = 9, 5, 3) and checked exhaustively around windows on
several grids: every staged row maps back to its slot, every other cell to
no slot."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROG = r'''
#define CPIC_PUSH_NS winmap
#include "push_impl.cuh"
#include <cstdio>
#include <vector>
using namespace cpic;
using namespace cpic::winmap;
int main() {
  long checked = 0, bad = 0;
  const int grids[][3] = {{16, 17, 9}, {64, 64, 64}, {128, 128, 128}, {7, 5, 4}, {96, 96, 64}};
  for (const auto& gd : grids) {
    const int sx = gd[0] + 2, sy = gd[1] + 2, sz = gd[2] + 2;
    const int ys = sx, zs = sx * sy, nc = sx * sy * sz;
    for (int wx : {3, 17, 44, 56, 64}) {
      if (wx > sx) continue;
      for (int c0 : {zs + ys + 1, nc / 2, nc - zs - ys - wx - 1}) {
        const TileWin w{c0, wx};
        const int lo = c0 - zs - ys - 8, hi = c0 + zs + ys + wx + 8;
        std::vector<int> expect(hi - lo, -1);
        for (int s = 0; s < kWinSeg; ++s)
          for (int x = 0; x < wx; ++x) {
            const int cell = segment_start(w, s, ys, zs) + x;
            if (cell < lo || cell >= hi || expect[cell - lo] != -1) { ++bad; continue; }  // overlap
            expect[cell - lo] = s * wx + x;
          }
        for (int cell = lo; cell < hi; ++cell) {
          ++checked;
          if (window_slot(cell, w, ys, zs) != expect[cell - lo]) ++bad;
        }
      }
    }
  }
  std::printf("%d %ld %ld\n", kWinSeg, checked, bad);
  return bad != 0;
}
'''


@pytest.mark.parametrize("shape", [9, 5, 3])
def test_window_slot_and_segment_start_agree(tmp_path, shape):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    src = tmp_path / "winmap.cu"
    src.write_text(PROG)
    exe = tmp_path / "winmap"
    r = subprocess.run([nvcc, "-std=c++17", "-O1", "-gencode", "arch=compute_103a,code=sm_103a",
                        f"-DCPIC_TILE_WINDOW={shape}", "-I", os.path.join(ROOT, "include"),
                        "-I", os.path.join(ROOT, "cabanapic_gb300", "csrc"), str(src), "-o", str(exe)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    segs, checked, bad = (int(t) for t in out.stdout.split())
    assert segs == shape and checked > 100000 and bad == 0
