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


U = 2.0 ** -53  # unit roundoff of FP64


def close_to_serial(got, ser, prod):
    """The GPU follows the reference's CUDA mode (--fmad=true): y = fma(p, q, s)
    where OCCA Serial rounds p*q first.  The two differ by at most the rounding of
    the product plus the final rounding of each: |got - ser| <= u (|pq| + |got| + |ser|)."""
    return np.all(np.abs(got - ser) <= U * (np.abs(prod) + np.abs(got) + np.abs(ser)))


@pytest.mark.parametrize("path", BS, ids=lambda p: p.stem)
def test_bs2_to_bs5_match_reference_values(cuda, orc, path):
    """BS2-BS5 on the GPU against the reference's own results (OCCA Serial, fixtures
    from its compiled sources): vectors within one rounding of the contracted
    product (the CUDA mode's fma, which the oracle's fmad=1 path matches bit for bit),
    the BS3/BS4/BS5 scalars within 1e-14 relative, for the order-exact kernels and
    for the integer-pipe BS3 that the drivers run by default."""
    from streamparanumal_gb300 import kernels as K

    g = json.loads(path.read_text())
    n, al, be = g["N"], g["alpha"], g["beta"]
    ha, hb = orc.uniform(n, g["seed"]), orc.uniform(n, g["seed"] + 1)
    a, b = torch.from_numpy(ha).cuda(), torch.from_numpy(hb).cuda()
    val = {k: float.fromhex(v) for k, v in g["value"].items()}
    # BS2: y = alpha a + beta b
    y = b.clone()
    K.bs2(n, al, a, be, y)
    ser = orc.bs2(al, ha, be, hb, fmad=0)
    assert sha(ser) == g["sha256"]["bs2"]                       # the checker is the reference
    got = y.cpu().numpy()
    np.testing.assert_array_equal(got, orc.bs2(al, ha, be, hb, fmad=1))
    assert close_to_serial(got, ser, al * ha)
    # BS3: order-exact, and the integer-pipe default
    tmp = torch.zeros(1024, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    nb = K.nblocks_for(n, 256)
    K.bs3_1(nb, n, a, tmp)
    K.bs3_2(nb, tmp, out)
    assert abs(out.item() - val["bs3"]) <= 1e-14 * val["bs3"]
    K.bs3_1_fast(nb, n, a, tmp, K.ReduceScratch())
    K.bs3_2(nb, tmp, out)
    assert abs(out.item() - val["bs3"]) <= 1e-14 * val["bs3"]
    # BS4
    K.bs4_1(nb, n, a, b, tmp)
    K.bs4_2(nb, tmp, out)
    assert abs(out.item() - val["bs4"]) <= 1e-14 * abs(val["bs4"])
    # BS5 at the reference's block size 1024, and at 256: r = r + alpha Ap, r.r
    for bs, key in ((1024, "bs5"), (256, "bs5_256")):
        nb5 = K.nblocks_for(n, bs)
        r = b.clone()
        K.bs5_1(nb5, n, a, al, r, tmp, block_size=bs)
        K.bs5_2(nb5, tmp, out, block_size=bs)
        assert abs(out.item() - val[key]) <= 1e-14 * val[key]
        if bs == 1024:
            r_ser, _, _ = orc.bs5(ha, al, hb, bs=1024, fmad=0)
            assert sha(r_ser) == g["sha256"]["bs5_r"]
            assert close_to_serial(r.cpu().numpy(), r_ser, al * ha)
        # the drivers' default stage 1 (r.r on the integer pipe): the same r
        r2 = b.clone()
        K.bs5_1_fast(nb5, n, a, al, r2, tmp, K.ReduceScratch(), block_size=bs)
        K.bs5_2(nb5, tmp, out, block_size=bs)
        assert torch.equal(r2, r)
        assert abs(out.item() - val[key]) <= 1e-14 * val[key]
