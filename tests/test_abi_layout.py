"""The ctypes mirrors in hnswgpu.py match include/hnswgpu.h: the size of every
struct and the offset of every field, read from a C program compiled against
the header (the structs gain fields at their ends as options are added)."""
from __future__ import annotations

import ctypes
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]


def test_ctypes_structs_match_the_c_header(hg, tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    pairs = [(hg._Filter, "hg_filter"), (hg._BatchOptions, "hg_batch_options"),
             (hg._ServerConfig, "hg_server_config"), (hg._Request, "hg_request"),
             (hg._ServerStats, "hg_server_stats"), (hg._BuildOptions, "hg_build_options")]
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "hnswgpu.h"', "int main(void) {"]
    for py, c in pairs:
        lines.append(f'  printf("{c} size %zu\\n", sizeof({c}));')
        for name, _ in py._fields_:
            lines.append(f'  printf("{c} {name} %zu\\n", offsetof({c}, {name}));')
    lines.append('  printf("hg_neighbor size %zu\\n", sizeof(hg_neighbor));')
    for name in ("label", "distance"):
        lines.append(f'  printf("hg_neighbor {name} %zu\\n", offsetof(hg_neighbor, {name}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", f"-I{REPO / 'include'}", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    got = {}
    for line in out.splitlines():
        c, name, val = line.split()
        got[(c, name)] = int(val)
    for py, c in pairs:
        assert ctypes.sizeof(py) == got[(c, "size")], c
        for name, _ in py._fields_:
            assert getattr(py, name).offset == got[(c, name)], (c, name)
    rec = np.dtype(hg.NEIGHBOR)
    assert rec.itemsize == got[("hg_neighbor", "size")]
    assert rec.fields["label"][1] == got[("hg_neighbor", "label")]
    assert rec.fields["distance"][1] == got[("hg_neighbor", "distance")]
