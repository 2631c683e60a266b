"""Batched persistent launch and graph capture (GPU): every instance gets the
oracle's x, r and q bits (the reference's fma update and its CSR-order
gather+scatter on the oracle's own ogs Setup of the same ids), the same bits as the
one-instance entry points, and r.r within 1e-14 relative of the double-double
oracle."""
import numpy as np
import pytest
import torch

from streamparanumal_gb300 import batch as B
from streamparanumal_gb300 import kernels as K
from streamparanumal_gb300 import ogs as O

pytestmark = pytest.mark.gpu


def instances(orc, count, seed, emax=5, pmax=5, with_ids=False):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        ex, ey, ez = (int(v) for v in rng.integers(2, emax + 1, size=3))
        p = int(rng.integers(2, pmax + 1))
        ids = O.box_hex_ids(ex, ey, ez, p, int(rng.integers(0, 3)))
        hids = ids.copy()
        h = O.ogs_t()
        h.Setup(ids.size, ids, unique=True)
        n = ids.size
        vec = {k: torch.from_numpy(orc.uniform(n, 100 * i + j)).cuda()
               for j, k in enumerate(("x", "r", "p", "Ap", "q"))}
        out.append((h, vec, 0.1 + 0.01 * i, hids) if with_ids else (h, vec, 0.1 + 0.01 * i))
    return out


def test_batch_matches_oracle_and_single_instance_calls(cuda, orc):
    inst = instances(orc, 7, 3, with_ids=True)
    ref = []
    sc = K.ReduceScratch()
    for h, v, alpha, hids in inst:
        x, r, q = v["x"].clone(), v["r"].clone(), v["q"].clone()
        rr = torch.zeros(1, dtype=torch.float64, device="cuda")
        K.cg_update(alpha, v["p"], v["Ap"], x, r, rr, sc)
        h.GatherScatter(q, 1, O.Add, O.Sym)
        xo, ro, rro = orc.cg_update(alpha, v["p"].cpu().numpy(), v["Ap"].cpu().numpy(),
                                    v["x"].cpu().numpy(), v["r"].cpu().numpy())
        csr = orc.ogs_setup(hids, kind=1, unique=True)
        qo = orc.gather_scatter(csr["rsT"], csr["ciT"], csr["rsT"], csr["ciT"],
                                v["q"].cpu().numpy())
        ref.append((x, r, q, rro, xo, ro, qo))
    inst = [(h, v, a) for h, v, a, _ in inst]
    rdotr = [torch.zeros(1, dtype=torch.float64, device="cuda") for _ in inst]
    b = B.Batch([h for h, _, _ in inst], [v["x"] for _, v, _ in inst],
                [v["r"] for _, v, _ in inst], [v["p"] for _, v, _ in inst],
                [v["Ap"] for _, v, _ in inst], rdotr, [v["q"] for _, v, _ in inst],
                [a for _, _, a in inst])
    b.run()
    torch.cuda.synchronize()
    for (h, v, _), (x, r, q, rro, xo, ro, qo), rd in zip(inst, ref, rdotr):
        np.testing.assert_array_equal(v["x"].cpu().numpy(), xo)
        np.testing.assert_array_equal(v["r"].cpu().numpy(), ro)
        np.testing.assert_array_equal(v["q"].cpu().numpy(), qo)
        assert torch.equal(v["x"], x) and torch.equal(v["r"], r) and torch.equal(v["q"], q)
        # tiles of 8192 entries (lane chains of 32 fma), tile partials in order
        assert abs(rd.item() - rro) <= 1e-14 * rro


def test_batch_graph_replay_and_repeat(cuda, orc):
    inst = instances(orc, 4, 11)
    rdotr = [torch.zeros(1, dtype=torch.float64, device="cuda") for _ in inst]
    args = ([h for h, _, _ in inst], [v["x"] for _, v, _ in inst], [v["r"] for _, v, _ in inst],
            [v["p"] for _, v, _ in inst], [v["Ap"] for _, v, _ in inst], rdotr,
            [v["q"] for _, v, _ in inst], [0.0 for _ in inst])  # alpha 0: x, r unchanged
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        b = B.Batch(*args, stream=s)
        b.run(stream=s)
        first = [t.item() for t in rdotr]
        g = B.Graph(s)
        with g:
            b.run(stream=s)
        for _ in range(3):
            g.launch()
    torch.cuda.synchronize()
    assert [t.item() for t in rdotr] == first  # tickets were reset; same order, same bits


def test_batch_fp32_storage_matches_single_instance_calls(cuda, orc):
    """FP32 storage: x, r and q equal to the oracle's FP32 update and FP32
    CSR-order gather+scatter, and bit-identical to the FP32 one-instance calls; r.r
    (compensated FP32 partials, FP64 finish) within 1e-12 of the exact sum of the
    FP32 r values' squares."""
    inst = [(h, {k: t.float() for k, t in v.items()}, a, hids)
            for h, v, a, hids in instances(orc, 6, 29, with_ids=True)]
    ref = []
    sc = K.ReduceScratch()
    for h, v, alpha, hids in inst:
        x, r, q = v["x"].clone(), v["r"].clone(), v["q"].clone()
        rr = torch.zeros(1, dtype=torch.float64, device="cuda")
        K.cg_update(alpha, v["p"], v["Ap"], x, r, rr, sc)
        h.GatherScatter(q, 1, O.Add, O.Sym)
        xo, ro, _ = orc.cg_update(np.float32(alpha), v["p"].cpu().numpy(),
                                  v["Ap"].cpu().numpy(), v["x"].cpu().numpy(),
                                  v["r"].cpu().numpy())
        csr = orc.ogs_setup(hids, kind=1, unique=True)
        qo = orc.gather_scatter(csr["rsT"], csr["ciT"], csr["rsT"], csr["ciT"],
                                v["q"].cpu().numpy())
        np.testing.assert_array_equal(x.cpu().numpy(), xo)
        np.testing.assert_array_equal(r.cpu().numpy(), ro)
        np.testing.assert_array_equal(q.cpu().numpy(), qo)
        ref.append((x, r, q))
    inst = [(h, v, a) for h, v, a, _ in inst]
    rdotr = [torch.zeros(1, dtype=torch.float64, device="cuda") for _ in inst]
    b = B.Batch([h for h, _, _ in inst], [v["x"] for _, v, _ in inst],
                [v["r"] for _, v, _ in inst], [v["p"] for _, v, _ in inst],
                [v["Ap"] for _, v, _ in inst], rdotr, [v["q"] for _, v, _ in inst],
                [a for _, _, a in inst])
    b.run()
    torch.cuda.synchronize()
    for (h, v, _), (x, r, q), rd in zip(inst, ref, rdotr):
        assert torch.equal(v["x"], x) and torch.equal(v["r"], r) and torch.equal(v["q"], q)
        exact = float(np.sum(r.cpu().numpy().astype(np.float64) ** 2))
        assert abs(rd.item() - exact) <= 1e-12 * exact


def test_batch_rejects_mixed_types(cuda, orc):
    (h, v, a), = instances(orc, 1, 5)
    rd = [torch.zeros(1, dtype=torch.float64, device="cuda")]
    with pytest.raises(TypeError):
        B.Batch([h], [v["x"].float()], [v["r"]], [v["p"]], [v["Ap"]], rd, [v["q"]], [a])


@pytest.mark.parametrize("order,rows", [(2, 0), (2, 1), (0, 0)])
def test_batch_with_every_chunk_walk(cuda, orc, order, rows):
    """Plans whose chunks walk renumbered, grouped or plain rows: the batch gives the
    one-instance bits."""
    from streamparanumal_gb300 import capi
    old = {k: capi.tune_get(k) for k in ("ogs.order", "ogs.rows")}
    try:
        capi.tune_set("ogs.order", order)
        capi.tune_set("ogs.rows", rows)
        inst = instances(orc, 4, 41)
    finally:
        for k, v in old.items():
            capi.tune_set(k, v)
    ref = []
    for h, v, alpha in inst:
        q = v["q"].clone()
        h.GatherScatter(q, 1, O.Add, O.Sym)
        ref.append(q)
    rdotr = [torch.zeros(1, dtype=torch.float64, device="cuda") for _ in inst]
    b = B.Batch([h for h, _, _ in inst], [v["x"] for _, v, _ in inst],
                [v["r"] for _, v, _ in inst], [v["p"] for _, v, _ in inst],
                [v["Ap"] for _, v, _ in inst], rdotr, [v["q"] for _, v, _ in inst],
                [a for _, _, a in inst])
    b.run()
    torch.cuda.synchronize()
    for (h, v, _), q in zip(inst, ref):
        assert torch.equal(v["q"], q)
