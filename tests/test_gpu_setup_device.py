"""ogs setup on the device (sp_ogs_setup_device) and box-mesh ids on the device
(sp_mesh_box_hex_ids_device) against their host forms and the oracle (GPU)."""
import numpy as np
import pytest
import torch

from streamparanumal_gb300 import capi
from streamparanumal_gb300 import ogs as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("box", [(1, 1, 1, 1, 0), (3, 4, 5, 2, 0), (4, 3, 2, 7, 99),
                                 (6, 5, 4, 3, 2024), (2, 7, 3, 5, 1)])
def test_box_ids_device_matches_host(cuda, box):
    nx, ny, nz, p, seed = box
    want = O.box_hex_ids(nx, ny, nz, p, seed)
    got = O.box_hex_ids(nx, ny, nz, p, seed, device="cuda")
    torch.cuda.synchronize()
    np.testing.assert_array_equal(got.cpu().numpy(), want)


def random_ids(n, seed, zeros=0.05, flagged=0.3, kmax=None):
    rng = np.random.default_rng(seed)
    keys = rng.integers(1, kmax or max(2, n // 3), size=n).astype(np.int64)
    keys[rng.random(n) < zeros] = 0
    keys[rng.random(n) < flagged] *= -1
    return keys


CASES = [
    ("box", lambda: O.box_hex_ids(5, 4, 3, 7, 2024)),
    ("box-lex", lambda: O.box_hex_ids(6, 3, 4, 3, 0)),
    ("random", lambda: random_ids(20000, 1)),
    ("random-big-keys", lambda: random_ids(5000, 2, kmax=1 << 40)),
    ("large-groups", lambda: np.repeat(np.arange(1, 41), 300).astype(np.int64)[
        np.random.default_rng(3).permutation(12000)]),
    ("all-ignored", lambda: np.zeros(100, dtype=np.int64)),
    ("singletons", lambda: np.arange(1, 3001, dtype=np.int64)),
]


@pytest.mark.parametrize("name,make_ids", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("kind,unique", [(capi.SIGNED, True), (capi.SIGNED, False),
                                         (capi.UNSIGNED, False)])
def test_setup_device_matches_host(cuda, orc, name, make_ids, kind, unique):
    ids = make_ids()
    if kind == capi.UNSIGNED:
        ids = np.abs(ids)
    h_host = O.ogs_t()
    ids_host = ids.copy()
    h_host.Setup(ids.size, ids_host, kind=kind, unique=unique)
    h_dev = O.ogs_t()
    d_ids = torch.from_numpy(ids.copy()).cuda()
    h_dev.Setup(ids.size, d_ids, kind=kind, unique=unique)
    torch.cuda.synchronize()
    # the same signs written back, the same plan
    np.testing.assert_array_equal(d_ids.cpu().numpy(), ids_host)
    assert h_dev.NgatherGlobal == h_host.NgatherGlobal
    assert h_dev.info.NrowsT == h_host.info.NrowsT and h_dev.info.nnzN == h_host.info.nnzN
    for trans in (O.Trans, O.NoTrans):
        rs_d, ci_d = h_dev.csr(trans)
        rs_h, ci_h = h_host.csr(trans)
        np.testing.assert_array_equal(rs_d, rs_h)
        np.testing.assert_array_equal(ci_d, ci_h)
    # and the oracle's
    ref = orc.ogs_setup(ids.copy(), kind=kind, unique=unique)
    rs_d, ci_d = h_dev.csr(O.Trans)
    np.testing.assert_array_equal(rs_d, ref["rsT"])
    np.testing.assert_array_equal(ci_d, ref["ciT"])
    h_host.Free()
    h_dev.Free()


def test_device_plan_gather_scatter_bit_exact(cuda, orc):
    """A plan built entirely on the device (ids and setup) gives the reference's bits."""
    d_ids = O.box_hex_ids(6, 5, 4, 7, 77, device="cuda")
    ids = d_ids.cpu().numpy()
    ref = orc.ogs_setup(ids.copy(), kind=capi.SIGNED, unique=True)
    h = O.ogs_t()
    h.Setup(d_ids.numel(), d_ids, kind=capi.SIGNED, unique=True)
    q = orc.uniform(ids.size, 19)
    dq = torch.from_numpy(q).cuda()
    h.GatherScatter(dq, 1, O.Add, O.Sym)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(
        dq.cpu().numpy(), orc.gather_scatter(ref["rsT"], ref["ciT"], ref["rsT"], ref["ciT"], q))
    h.Free()


def test_setup_device_rejects_bad_arguments(cuda):
    h = O.ogs_t()
    d_ids = torch.ones(10, dtype=torch.int64, device="cuda")
    with pytest.raises(capi.SpError, match="Invalid ogs setup requested"):
        h.Setup(10, d_ids, kind=capi.UNSIGNED, unique=True)
    with pytest.raises(TypeError):
        h.Setup(10, d_ids.to(torch.int32))
    with pytest.raises(ValueError):
        h.Setup(11, d_ids)
