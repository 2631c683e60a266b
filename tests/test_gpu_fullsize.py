"""Parity at the benchmark's full sizes (GPU): BS1-BS5 at N = 2^28 and BS6-BS8 on
the permuted 64^3 p = 7 box (134,217,728 local nodes), through properties that do
not need the oracle to run the whole workload:

* elementwise kernels (copy, axpy, the BS5 update of r) against the oracle on a
  strided sample of entries -- each entry is computed independently, so the
  sample is exact;
* the order-exact reductions against the oracle's restatement of the reference's
  partition on the full vectors (it runs in a few seconds with OpenMP);
* the integer-pipe BS3 norm (the drivers' default) within 1e-14 relative of the
  order-exact result and within 4 ulps of the double-double sum, on the full
  vector;
* on the permuted 64^3 p = 7 box: the device-built ids and CSR equal to the
  oracle's (the reference's min-propagation ids and ogs Setup restated, run on
  the host with OpenMP), and BS6, BS7 and BS8 equal bit for bit to the oracle's
  loops on the same inputs; plus gather+scatter against gather then scatter and
  multiplicities from a gather of ones.
"""
import hashlib

import numpy as np
import pytest
import torch

from streamparanumal_gb300 import kernels as K
from streamparanumal_gb300 import ogs as O

pytestmark = pytest.mark.gpu

N = 1 << 28
STRIDE = 4099


def test_bs1_bs2_bs5_full_length_sampled(cuda, orc):
    a = torch.from_numpy(orc.uniform(N, 11)).cuda()
    b = torch.from_numpy(orc.uniform(N, 12)).cuda()
    y = torch.empty_like(a)
    K.bs1(N, a, y)
    assert torch.equal(y, a)
    alpha, beta = -0.7353, 0.4142
    y.copy_(b)
    K.bs2(N, alpha, a, beta, y)
    idx = torch.arange(0, N, STRIDE, device="cuda")
    want = orc.bs2(alpha, a[idx].cpu().numpy(), beta, b[idx].cpu().numpy(), fmad=1)
    np.testing.assert_array_equal(y[idx].cpu().numpy(), want)
    del y
    # BS5 (reference block size 1024): r of the sample, r.r of the whole vector
    nb = K.nblocks_for(N, 1024)
    r = b.clone()
    tmp = torch.zeros(1024, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    K.bs5_1(nb, N, a, alpha, r, tmp, block_size=1024)
    K.bs5_2(nb, tmp, out, block_size=1024)
    r_ref, part, res = orc.bs5(a.cpu().numpy(), alpha, b.cpu().numpy(), bs=1024, nblocks=nb,
                               fmad=1)
    np.testing.assert_array_equal(r[idx].cpu().numpy(), r_ref[idx.cpu().numpy()])
    np.testing.assert_array_equal(tmp[:nb].cpu().numpy(), part)
    assert out.item() == res


def test_bs3_bs4_full_length_order_exact(cuda, orc):
    ha, hb = orc.uniform(N, 21), orc.uniform(N, 22)
    a, b = torch.from_numpy(ha).cuda(), torch.from_numpy(hb).cuda()
    nb = K.nblocks_for(N, 256)
    tmp = torch.zeros(256, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    K.bs3_1(nb, N, a, tmp)
    K.bs3_2(nb, tmp, out)
    part, res = orc.bs3(ha, bs=256, nblocks=nb, fmad=1)
    np.testing.assert_array_equal(tmp[:nb].cpu().numpy(), part)
    assert out.item() == res
    K.bs4_1(nb, N, a, b, tmp)
    K.bs4_2(nb, tmp, out)
    part, res = orc.bs4(ha, hb, bs=256, nblocks=nb, fmad=1)
    np.testing.assert_array_equal(tmp[:nb].cpu().numpy(), part)
    assert out.item() == res


def test_bs3_fast_norm_full_length(cuda, orc):
    ha = orc.uniform(N, 21)
    a = torch.from_numpy(ha).cuda()
    nb = K.nblocks_for(N, 256)
    tmp = torch.full((256,), float("nan"), dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    K.bs3_1_fast(nb, N, a, tmp, K.ReduceScratch())
    K.bs3_2(nb, tmp, out)
    got = out.item()
    assert torch.all(tmp[1:nb] == 0)
    _, ref_order = orc.bs3(ha, bs=256, nblocks=nb, fmad=1)
    assert abs(got - ref_order) <= 1e-14 * ref_order
    exact = orc.dot_dd(ha, ha)
    assert abs(got - exact) <= 4 * np.spacing(exact)


def sha(x):
    return hashlib.sha256(np.ascontiguousarray(x).tobytes()).hexdigest()


def test_ogs_full_size_permuted_box(cuda, orc):
    E, p, seed = 64, 7, 20240607
    ids = O.box_hex_ids(E, E, E, p, seed, device="cuda")
    Nt = ids.numel()
    # ids: the device lattice formula against the oracle's min-propagation
    hids = orc.box_hex_ids(E, E, E, p, seed)
    assert sha(ids.cpu().numpy()) == sha(hids)
    h = O.ogs_t()
    h.Setup(Nt, ids, unique=True)
    del ids
    Ng = h.NgatherGlobal
    # the device-built T operator against the oracle's ogs Setup (rows in order of
    # first appearance, columns ascending: ogsSetup.cpp:492-579)
    ref = orc.ogs_setup(hids, kind=1, unique=True)
    del hids
    rs, ci = h.csr(O.Trans)
    assert sha(rs) == sha(ref["rsT"]) and sha(ci) == sha(ref["ciT"])
    del ref
    # BS6 / BS7 / BS8 on the full box against the oracle's loops, bit for bit
    hq = orc.uniform(Nt, 41)
    q = torch.from_numpy(hq).cuda()
    gq = torch.empty(Ng, dtype=torch.float64, device="cuda")
    h.Gather(gq, q, 1, O.Add, O.Trans)
    want_g = orc.gather(rs, ci, hq)
    assert sha(gq.cpu().numpy()) == sha(want_g)
    hgv = orc.uniform(Ng, 42)
    out = torch.zeros(Nt, dtype=torch.float64, device="cuda")
    h.Scatter(out, torch.from_numpy(hgv).cuda(), 1, O.NoTrans)
    assert sha(out.cpu().numpy()) == sha(orc.scatter(rs, ci, hgv, np.zeros(Nt)))
    del out, hgv
    h.GatherScatter(q, 1, O.Add, O.Sym)
    assert sha(q.cpu().numpy()) == sha(orc.gather_scatter(rs, ci, rs, ci, hq))
    del q, gq, want_g, hq, rs, ci
    torch.cuda.empty_cache()
    assert Ng == (E * p + 1) ** 3
    # multiplicities: a gather of ones counts each row's members (1, 2, 4 or 8)
    ones = torch.ones(Nt, dtype=torch.float64, device="cuda")
    mult = torch.empty(Ng, dtype=torch.float64, device="cuda")
    h.Gather(mult, ones, 1, O.Add, O.Trans)
    assert float(mult.sum()) == Nt
    assert set(torch.unique(mult).cpu().tolist()) == {1.0, 2.0, 4.0, 8.0}
    del ones
    # gather+scatter == scatter(gather): the same CSR-order sums, bit for bit
    q = torch.from_numpy(orc.uniform(Nt, 31)).cuda()
    gq = torch.empty(Ng, dtype=torch.float64, device="cuda")
    h.Gather(gq, q, 1, O.Add, O.Trans)
    via = torch.empty_like(q)
    h.Scatter(via, gq, 1, O.NoTrans)
    gs = q.clone()
    h.GatherScatter(gs, 1, O.Add, O.Sym)
    assert torch.equal(gs, via)
