"""include/cpic/layout.h (the layouts a C or C++ caller binds to) against the
Python mirror in cabanapic_gb300/layout.py: a C program built from the
header prints sizes, cell AoSoA offsets, particle member offsets and voxel
indices, and the Python packers must put each value where the header says."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from cabanapic_gb300 import layout as L

ROOT_INCLUDE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")

_C = r"""
#include <stdio.h>
#include "cpic/layout.h"
/* particle member m of particle p: the SoA block of the header's comment */
static size_t particle_byte_offset(int64_t p, int m, int rb, int vl) {
  size_t base = (size_t)(p / vl) * cpic_particle_block_bytes(rb, vl);
  size_t lane = (size_t)(p % vl);
  return m < 7 ? base + (size_t)m * vl * rb + lane * rb : base + (size_t)7 * vl * rb + lane * 4;
}
int main(void) {
  int rbs[2] = {4, 8}, vls[2] = {16, 32};
  long long ns[5] = {0, 1, 31, 33, 1000};
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b) {
      for (int k = 0; k < 5; ++k)
        printf("plist %d %d %lld %zu\n", rbs[a], vls[b], ns[k], cpic_particle_list_bytes(ns[k], rbs[a], vls[b]));
      for (long long p = 0; p < 70; p += 3)
        for (int m = 0; m < 8; ++m)
          printf("poff %d %d %lld %d %zu\n", rbs[a], vls[b], p, m, particle_byte_offset(p, m, rbs[a], vls[b]));
    }
  for (int a = 0; a < 2; ++a)
    for (int k = 0; k < 5; ++k) {
      printf("carr %d 9 %lld %zu\n", rbs[a], ns[k], cpic_cell_array_bytes(ns[k], 9, rbs[a]));
      printf("carr %d 18 %lld %zu\n", rbs[a], ns[k], cpic_cell_array_bytes(ns[k], 18, rbs[a]));
    }
  for (long long c = 0; c < 100; c += 7)
    for (int m = 0; m < 18; m += 5) printf("coff %lld 18 %d %zu\n", c, m, cpic_cell_offset(c, 18, m));
  for (long long c = 0; c < 100; c += 7)
    for (int m = 0; m < 9; m += 4) printf("coff %lld 9 %d %zu\n", c, m, cpic_cell_offset(c, 9, m));
  printf("vox %lld\n", (long long)cpic_voxel(3, 2, 5, 7, 4, 1));
  printf("vox %lld\n", (long long)cpic_voxel(0, 6, 1, 130, 130, 1));
  return 0;
}
"""


@pytest.fixture(scope="module")
def header_lines(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("layout")
    src, exe = d / "layout.c", d / "layout"
    src.write_text(_C)
    subprocess.run([cc, "-std=c99", "-O1", "-I", ROOT_INCLUDE, "-o", str(exe), str(src)], check=True)
    return subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines()


def _real(rb):
    return np.float32 if rb == 4 else np.float64


def test_sizes_match(header_lines):
    for ln in header_lines:
        t = ln.split()
        if t[0] == "plist":
            rb, vl, n, v = map(int, t[1:])
            assert L.particle_list_bytes(n, _real(rb), vl) == v, ln
        elif t[0] == "carr":
            rb, m, n, v = map(int, t[1:])
            assert L.cell_array_bytes(n, m, _real(rb)) == v, ln


def test_particle_packer_puts_members_at_the_header_offsets(header_lines):
    n = 70
    for rb in (4, 8):
        R = _real(rb)
        for vl in (16, 32):
            p = {k: (np.arange(n) * 10 + i).astype(R) for i, k in enumerate(("x", "y", "z", "ux", "uy", "uz", "w"))}
            p["cell"] = (np.arange(n) * 10 + 7).astype(np.int32)
            raw = L.pack_particles(p, R, vl).view(np.uint8)
            for ln in header_lines:
                t = ln.split()
                if t[0] != "poff" or int(t[1]) != rb or int(t[2]) != vl:
                    continue
                pi, m, off = int(t[3]), int(t[4]), int(t[5])
                dt = np.int32 if m == 7 else R
                val = raw[off: off + np.dtype(dt).itemsize].view(dt)[0]
                assert val == pi * 10 + m, ln


def test_cell_packer_and_voxel_match(header_lines):
    for members in (9, 18):
        nc = 100
        vals = (np.arange(nc)[:, None] * 100 + np.arange(members)[None, :]).astype(np.float64)
        flat = L.pack_cells(vals, np.float64)
        for ln in header_lines:
            t = ln.split()
            if t[0] == "coff" and int(t[2]) == members:
                c, m, off = int(t[1]), int(t[3]), int(t[4])
                assert flat[off] == c * 100 + m, ln
    vox = [int(ln.split()[1]) for ln in header_lines if ln.startswith("vox")]
    assert vox == [L.voxel(3, 2, 5, 7, 4), L.voxel(0, 6, 1, 130, 130)]
