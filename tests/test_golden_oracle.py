"""The oracle reproduces the reference's own outputs (tests/golden, produced by the
reference's host code compiled from its sources; see tests/golden/make_golden.py).
CPU only: this pins the checker that every GPU parity test relies on."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden"
OGS = sorted(GOLD.glob("ogs_*.json"))
BS = sorted(GOLD.glob("bs_n*.json"))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def row_of(rs, ci, n):
    ro = np.full(n, -1, np.int64)
    for r in range(rs.size - 1):
        ro[ci[rs[r]:rs[r + 1]]] = r
    return ro


def test_fixtures_present():
    assert len(OGS) >= 6 and len(BS) >= 5


@pytest.mark.parametrize("path", OGS, ids=lambda p: p.stem)
def test_oracle_matches_reference_ogs(orc, path):
    g = json.loads(path.read_text())
    nx, ny, nz, p = g["mesh"]
    ids = orc.box_hex_ids(nx, ny, nz, p, g["perm_seed"])
    assert ids.size == g["N"]
    csr = orc.ogs_setup(ids.copy(), kind=1, unique=True)
    rs, ci = csr["rsT"], csr["ciT"]
    assert rs.size - 1 == g["Ngather"]
    if g["N"] <= 40000:
        assert sha(row_of(rs, ci, ids.size)) == g["sha256"]["abs_ids_rows"]
    q = orc.uniform(ids.size, g["qseed"])
    assert sha(q) == g["sha256"]["q"]
    assert sha(orc.gather_scatter(rs, ci, rs, ci, q)) == g["sha256"]["gs_sym"]
    assert sha(orc.gather(rs, ci, q)) == g["sha256"]["gather_trans"]
    gvals = orc.uniform(rs.size - 1, g["qseed"] + 1)
    assert sha(orc.scatter(rs, ci, gvals, np.zeros(ids.size))) == g["sha256"]["scatter_notrans"]
    if "ids_file" in g:
        # the reference's own owner choice, fed back as signed ids
        rid = np.load(GOLD / g["ids_file"])
        c2 = orc.ogs_setup(rid.copy(), kind=1, unique=False)
        np.testing.assert_array_equal(c2["rsT"], rs)
        np.testing.assert_array_equal(c2["ciT"], ci)
        assert sha(orc.gather(c2["rsN"], c2["ciN"], q)) == g["sha256"]["gather_notrans"]


@pytest.mark.parametrize("path", BS, ids=lambda p: p.stem)
def test_oracle_matches_reference_bs_serial(orc, path):
    """fmad=0 is OCCA Serial's separate multiply and add."""
    g = json.loads(path.read_text())
    n = g["N"]
    a = orc.uniform(n, g["seed"])
    b = orc.uniform(n, g["seed"] + 1)
    assert sha(a) == g["sha256"]["bs1"]
    assert sha(orc.bs2(g["alpha"], a, g["beta"], b, fmad=0)) == g["sha256"]["bs2"]
    part, res = orc.bs3(a, bs=256, fmad=0)
    assert sha(part) == g["sha256"]["bs3_partial"]
    assert res.hex() == g["value"]["bs3"]
    part, res = orc.bs4(a, b, bs=256, fmad=0)
    assert sha(part) == g["sha256"]["bs4_partial"]
    assert res.hex() == g["value"]["bs4"]
    r, part, res = orc.bs5(a, g["alpha"], b, bs=1024, fmad=0)
    assert sha(r) == g["sha256"]["bs5_r"]
    assert sha(part) == g["sha256"]["bs5_partial"]
    assert res.hex() == g["value"]["bs5"]
    _, _, res256 = orc.bs5(a, g["alpha"], b, bs=256, fmad=0)
    assert res256.hex() == g["value"]["bs5_256"]


@pytest.mark.parametrize("path", BS, ids=lambda p: p.stem)
def test_cuda_mode_contraction_stays_close_to_serial(orc, path):
    """The CUDA-mode (fmad) results differ from Serial mode only by the rounding of
    the contracted products: norm within 1e-14 relative."""
    g = json.loads(path.read_text())
    a = orc.uniform(g["N"], g["seed"])
    _, res = orc.bs3(a, bs=256, fmad=1)
    ref = float.fromhex(g["value"]["bs3"])
    assert abs(res - ref) <= 1e-14 * ref
