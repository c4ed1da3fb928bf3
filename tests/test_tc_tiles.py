"""The tile set and tile order of the tensor-core update (csrc/tc_tiles.h), built for the host
with g++: every tile of the update region -- one or two rectangles, or the lower triangle of a
square for the symmetric updates -- is visited exactly once, and the epilogue of a tile reads
exactly the 32-column chunks that hold columns of its rectangle."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "beast.jl_gb300", "csrc")

HARNESS = r"""
#include "tc_tiles.h"
extern "C" {
// the region of (m_rows, n_cols) x 2 and lower; out[4 t ..] = (r, m0, n0, valid) of tile t
int t_tiles(int mr0, int nc0, int mr1, int nc1, int lower, int cap, int* out) {
  TcRegion Rg = {};
  Rg.m_rows[0] = mr0; Rg.n_cols[0] = nc0; Rg.m_rows[1] = mr1; Rg.n_cols[1] = nc1;
  Rg.lower = lower;
  tc_region_count(Rg);
  if (Rg.ntiles > cap) return -1;
  for (int t = 0; t < Rg.ntiles; ++t) {
    int r, m0, n0;
    const bool v = tc_tile_at(Rg, t, r, m0, n0);
    out[4 * t] = r; out[4 * t + 1] = m0; out[4 * t + 2] = n0; out[4 * t + 3] = v ? 1 : 0;
  }
  return Rg.ntiles;
}
int t_chunks(int n_cols, int n0) { return tc_tile_chunks(n_cols, n0); }
}
"""


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("tctiles")
    src, so = d / "h.cpp", d / "h.so"
    src.write_text(HARNESS)
    subprocess.check_call(["g++", "-O2", "-shared", "-fPIC", "-I", CSRC, str(src), "-o", str(so)])
    L = C.CDLL(str(so))
    L.t_tiles.argtypes = [C.c_int] * 6 + [C.c_void_p]
    L.t_chunks.argtypes = [C.c_int, C.c_int]
    return L


def _visit(lib, mr0, nc0, mr1=0, nc1=0, lower=0):
    cap = 400000
    out = np.zeros(4 * cap, np.int32)
    n = lib.t_tiles(mr0, nc0, mr1, nc1, lower, cap, out.ctypes.data)
    assert n >= 0
    return out[:4 * n].reshape(n, 4)


# (real rows, complex columns) of C' as the LU's updates make them: in-block (N <= 192),
# mid-block (N = 256 .. 768), trailing squares of the lower triangle, odd sizes
RECTS = [(2 * 30656, 192), (2 * 30656, 64), (2 * 29952, 768), (2 * 77, 77), (2 * 1101, 300), (250, 1000),
         (2 * 5000, 256)]
SQUARES = [77, 300, 1576, 2640, 6656, 12345, 29696]


@pytest.mark.parametrize("mr,nc", RECTS)
def test_rectangle_tiles_visited_once(lib, mr, nc):
    v = _visit(lib, mr, nc)
    assert np.all(v[:, 3] == 1) and np.all(v[:, 0] == 0)
    got = {(int(m0), int(n0)) for _, m0, n0, _ in v}
    want = {(m * 128, k * 256) for m in range((mr + 127) // 128) for k in range(max(1, (nc + 255) // 256))}
    assert len(got) == len(v) and got == want


def test_two_rectangles_share_the_order(lib):
    """the L-shaped update: rectangle 0 (all rows, the block's columns) first, then rectangle 1
    (the block's rows, the columns beyond it)"""
    v = _visit(lib, 2 * 4000, 448, 2 * 192, 2900)
    r = v[:, 0]
    assert np.all(np.diff(r) >= 0) and r[0] == 0 and r[-1] == 1
    for rr, (mr, nc) in enumerate([(2 * 4000, 448), (2 * 192, 2900)]):
        t = v[r == rr]
        got = {(int(m0), int(n0)) for _, m0, n0, _ in t}
        assert got == {(m * 128, k * 256) for m in range((mr + 127) // 128) for k in range((nc + 255) // 256)}


@pytest.mark.parametrize("m", SQUARES)
def test_lower_triangle_tiles_visited_once(lib, m):
    v = _visit(lib, 2 * m, m, lower=1)
    valid = v[v[:, 3] == 1]
    got = {(int(m0), int(n0)) for _, m0, n0, _ in valid}
    ntm, ntn = (2 * m + 127) // 128, (m + 255) // 256
    want = {(a * 128, b * 256) for a in range(ntm) for b in range(min(a // 4 + 1, ntn))}
    assert len(got) == len(valid) and got == want
    # every tile holds an element on or below the diagonal: its first column <= its last row
    assert np.all(valid[:, 2] <= (valid[:, 1] + 127) // 2)


def test_whole_groups_go_column_by_column(lib):
    """consecutive indices of a whole group of four row tiles share a column tile four at a time"""
    v = _visit(lib, 2 * 8192, 8192, lower=1)
    g = 20  # group 20: row tiles 80 .. 83, 21 column tiles, starting at tile 2 g (g + 1)
    t0 = 2 * g * (g + 1)
    grp = v[t0:t0 + 4 * (g + 1)]
    assert np.all(grp[:, 1] // 128 == 80 + np.arange(4 * (g + 1)) % 4)
    assert np.all(grp[:, 2] // 256 == np.arange(4 * (g + 1)) // 4)


def test_epilogue_chunks(lib):
    assert lib.t_chunks(192, 0) == 6 and lib.t_chunks(64, 0) == 2 and lib.t_chunks(256, 0) == 8
    assert lib.t_chunks(1000, 768) == 8 and lib.t_chunks(800, 768) == 1 and lib.t_chunks(77, 0) == 3
