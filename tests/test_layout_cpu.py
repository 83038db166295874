"""The element order of the compressed row copies (compressed_layout.cuh):
a bijection inside every 128-element chunk, inverse functions that agree,
and the property the tensor-core walk relies on -- thread t of an MMA quad
finds, at k-step s, the dims (16s + 2t, +1) in its register 2s and
(16s + 2t + 8, +9) in register 2s + 1 -- checked on the host by compiling the
header as plain C++."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]

PROGRAM = r"""
#include <cstdio>
#include <cstdint>
#include <set>
#define __host__
#define __device__
#include "compressed_layout.cuh"
int main() {
  int bad = 0;
  for (int prec = 1; prec <= 2; ++prec) {
    const uint32_t per16 = prec == 1 ? 8u : 16u;  // elements per 16-byte load
    for (uint32_t pdc : {128u, 256u, 1024u}) {
      std::set<uint32_t> seen;
      for (uint32_t k = 0; k < pdc; ++k) {
        const uint32_t p = hg::cl_pos(k, prec);
        if (p >= pdc || (p >> 7) != (k >> 7)) ++bad;
        if (hg::cl_logical(p, prec) != k) ++bad;
        seen.insert(p);
      }
      if (seen.size() != pdc) ++bad;
    }
    // thread t's 16-byte load i of a chunk holds stream elements e = per16*i .. +per16-1,
    // stored at positions i*4*per16 + t*per16 + (e % per16)
    for (uint32_t t = 0; t < 4; ++t)
      for (uint32_t e = 0; e < 32; ++e) {
        const uint32_t i = e / per16;
        const uint32_t p = i * 4 * per16 + t * per16 + (e % per16);
        const uint32_t k = hg::cl_logical(p, prec);
        const uint32_t s = e / 4, w = e % 4;  // register 2s + (w >> 1), half (w & 1)
        const uint32_t want = 16 * s + 2 * t + 8 * (w >> 1) + (w & 1);
        if (k != want) ++bad;
      }
  }
  std::printf("%d\n", bad);
  return bad != 0;
}
"""


def test_compressed_layout(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "layout.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "layout"
    subprocess.run([cxx, "-std=c++17", f"-I{REPO / 'hnsw-engine_gb300' / 'csrc'}", str(src), "-o", str(exe)],
                   check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
