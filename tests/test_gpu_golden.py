"""The CUDA kernels reproduce the reference's own outputs (tests/golden) bit for
bit: BS6 gather, BS7 scatter and BS8 gather+scatter on hex boxes (lexicographic and
permuted elements, including the 16x16x16 p=7 anchor case), the N-operator gather
with the reference's own owner flags, and BS1 copy (GPU)."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest
import torch

from streamparanumal_gb300 import ogs as O

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"
OGS = sorted(GOLD.glob("ogs_*.json"))
BS = sorted(GOLD.glob("bs_n*.json"))


def sha(t):
    torch.cuda.synchronize()
    a = t.cpu().numpy() if isinstance(t, torch.Tensor) else t
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("path", OGS, ids=lambda p: p.stem)
def test_ogs_kernels_match_reference(cuda, orc, path):
    g = json.loads(path.read_text())
    nx, ny, nz, p = g["mesh"]
    ids = O.box_hex_ids(nx, ny, nz, p, g["perm_seed"])
    h = O.ogs_t()
    h.Setup(ids.size, ids, kind=O.Signed, unique=True)
    assert h.NgatherGlobal == g["Ngather"]
    q = torch.from_numpy(orc.uniform(ids.size, g["qseed"])).cuda()
    gq = torch.zeros(h.Ngather, dtype=torch.float64, device="cuda")
    h.Gather(gq, q, 1, O.Add, O.Trans)                       # BS6
    assert sha(gq) == g["sha256"]["gather_trans"]
    gv = torch.from_numpy(orc.uniform(h.Ngather, g["qseed"] + 1)).cuda()
    qs = torch.zeros(ids.size, dtype=torch.float64, device="cuda")
    h.Scatter(qs, gv, 1, O.NoTrans)                          # BS7
    assert sha(qs) == g["sha256"]["scatter_notrans"]
    h.GatherScatter(q, 1, O.Add, O.Sym)                      # BS8
    assert sha(q) == g["sha256"]["gs_sym"]
    if "ids_file" in g:
        rid = np.load(GOLD / g["ids_file"]).astype(np.int64)
        h2 = O.ogs_t()
        h2.Setup(rid.size, rid.copy(), kind=O.Signed, unique=False)
        q = torch.from_numpy(orc.uniform(rid.size, g["qseed"])).cuda()
        gq = torch.zeros(h2.Ngather, dtype=torch.float64, device="cuda")
        h2.Gather(gq, q, 1, O.Add, O.NoTrans)
        assert sha(gq) == g["sha256"]["gather_notrans"]


@pytest.mark.parametrize("path", BS, ids=lambda p: p.stem)
def test_bs1_matches_reference(cuda, orc, path):
    from streamparanumal_gb300 import kernels as K

    g = json.loads(path.read_text())
    a = torch.from_numpy(orc.uniform(g["N"], g["seed"])).cuda()
    b = torch.empty_like(a)
    K.bs1(g["N"], a, b)
    assert sha(b) == g["sha256"]["bs1"]
