"""The lane-row slab layout of kernel 7 on the host (no GPU): build_slabs,
compress_slabs and compress_slab_rows (streamparanumal_gb300/csrc/sp_ogs_order.cpp)
are compiled with a
checker (tests/native/slab_layout_check.cpp) that walks every slab the way the
kernel's index arithmetic does -- full passes of 8 and 16 members per lane, the
row steps of a slab's rest, any row size, 16-bit codes decoded through the slab's
table, row codes through the slab's row table -- checks every index against its
array and the results against the CSR-order sums bit for bit, for the gather and
the in-place gather+scatter."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from streamparanumal_gb300 import ogs as O

ROOT = Path(__file__).resolve().parent.parent
CSRC = ROOT / "streamparanumal_gb300" / "csrc"


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    from streamparanumal_gb300 import _build
    out = tmp_path_factory.mktemp("slabs") / "slab_layout_check"
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", f"-I{CSRC}", f"-I{ROOT / 'include'}",
           f"-I{_build._cuda_home() / 'include'}", str(ROOT / "tests" / "native" /
                                                       "slab_layout_check.cpp"),
           str(CSRC / "sp_ogs_order.cpp"), "-o", str(out)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-3000:]
    return out


def run(checker, tmp_path, rs, ci, n, order=1, page=9, ball=0, seg=14, shift=0, row_seed=0):
    (tmp_path / "rs.bin").write_bytes(np.ascontiguousarray(rs, dtype=np.int32).tobytes())
    (tmp_path / "ci.bin").write_bytes(np.ascontiguousarray(ci, dtype=np.int32).tobytes())
    res = subprocess.run([str(checker), str(tmp_path / "rs.bin"), str(tmp_path / "ci.bin"),
                          str(n), str(order), str(page), str(ball), str(seg), str(shift),
                          str(row_seed)],
                         capture_output=True, text=True)
    assert res.returncode == 0 and res.stdout.startswith("ok"), res.stdout + res.stderr
    coded, total, rows_coded, nrows = (int(x) for x in res.stdout.split()[2::2])
    return coded, total, rows_coded, nrows


BOXES = [((2, 2, 2, 1, 0), 3), ((5, 4, 3, 7, 2024), 9), ((6, 6, 6, 2, 5), 5),
         ((9, 8, 7, 5, 3), 8), ((4, 3, 5, 3, 77), 6), ((8, 8, 8, 7, 11), 9)]


@pytest.mark.parametrize("box,shift", BOXES)
@pytest.mark.parametrize("order,seg", [(0, 14), (1, 8), (1, 17)])
def test_slab_layout_of_box_meshes(orc, checker, tmp_path, box, shift, order, seg):
    nx, ny, nz, p, seed = box
    ids = O.box_hex_ids(nx, ny, nz, p, seed)
    csr = orc.ogs_setup(ids.copy(), kind=1, unique=True)
    coded, total, rows_coded, nrows = run(checker, tmp_path, csr["rsT"], csr["ciT"], ids.size,
                                          order=order, seg=seg, shift=shift)
    # elements of (p+1)^3 <= 2^shift nodes: nearly every slab compresses, ids and rows
    assert total == 2 * ids.size and coded >= 0.6 * total
    assert nrows == csr["rsT"].size - 1 and rows_coded >= 0.6 * nrows


@pytest.mark.parametrize("seg,shift", [(8, 0), (8, 9), (14, 12), (14, 3)])
def test_slab_layout_any_row_size_and_empty_rows(orc, checker, tmp_path, seg, shift):
    rng = np.random.default_rng(21)
    sizes = rng.integers(0, 41, size=2500)
    n = int(sizes.sum())
    rs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int32)
    ci = rng.permutation(n).astype(np.int32)
    run(checker, tmp_path, rs, ci, n, order=0, seg=seg, shift=shift)


@pytest.mark.parametrize("box,shift", [((5, 4, 3, 7, 2024), 9), ((6, 6, 6, 2, 5), 5)])
def test_slab_row_words_beyond_the_row_table(orc, checker, tmp_path, box, shift):
    """Row words that a seeded permutation scatters over the whole row range: a slab
    whose rows fall into more than 32 runs (or whose codes do not fit 16 bits)
    keeps its 32-bit row words, the others decode through their row table, and the
    gather still lands every row's sum on its permuted row word."""
    nx, ny, nz, p, seed = box
    ids = O.box_hex_ids(nx, ny, nz, p, seed)
    csr = orc.ogs_setup(ids.copy(), kind=1, unique=True)
    rs, ci = csr["rsT"], csr["ciT"]
    _, _, rows_sorted, nrows = run(checker, tmp_path, rs, ci, ids.size, shift=shift)
    _, _, rows_perm, nrows_p = run(checker, tmp_path, rs, ci, ids.size, shift=shift, row_seed=17)
    assert nrows == nrows_p == rs.size - 1
    # first-appearance rows fall into few runs; permuted ones mostly do not
    assert rows_sorted >= 0.6 * nrows and rows_perm < 0.5 * nrows
