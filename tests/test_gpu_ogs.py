"""ogs gather / scatter / gather+scatter kernels against the oracle's host loops
(GPU).  Every type, op and transpose is bit-exact: sums run in CSR order from the
op's identity, exactly as ogsOperator_t's loops do."""
import numpy as np
import pytest
import torch

from streamparanumal_gb300 import capi
from streamparanumal_gb300 import ogs as O

pytestmark = pytest.mark.gpu

NP_TYPES = {capi.FLOAT: np.float32, capi.DOUBLE: np.float64, capi.INT32: np.int32,
            capi.INT64: np.int64}


def values(orc, n, dtype, seed):
    u = orc.uniform(n, seed)
    if dtype in (np.float32, np.float64):
        return u.astype(dtype)
    return np.round(u * 1000).astype(dtype)


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def pad(rs, nrows):
    return np.concatenate([rs, np.full(nrows + 1 - rs.size, rs[-1], rs.dtype)])


def make(orc, ids, kind=capi.SIGNED, unique=True):
    ids_o = ids.copy()
    ref = orc.ogs_setup(ids_o, kind=kind, unique=unique)
    h = O.ogs_t()
    ids_p = ids.copy()
    h.Setup(ids.size, ids_p, kind=kind, unique=unique)
    rsT, ciT = h.csr(O.Trans)
    np.testing.assert_array_equal(rsT, ref["rsT"])
    np.testing.assert_array_equal(ciT, ref["ciT"])
    return h, ref


BOXES = [(2, 2, 2, 1, 0), (3, 2, 2, 3, 0), (4, 3, 2, 2, 99), (4, 4, 4, 7, 0), (5, 4, 3, 7, 2024),
         (16, 16, 16, 7, 0)]


@pytest.mark.parametrize("box", BOXES)
def test_box_gather_scatter_sym_fp64(cuda, orc, box):
    nx, ny, nz, p, seed = box
    ids = O.box_hex_ids(nx, ny, nz, p, seed)
    h, ref = make(orc, ids)
    q = orc.uniform(ids.size, 17)
    dq = torch.from_numpy(q).cuda()
    h.GatherScatter(dq, 1, O.Add, O.Sym)
    want = orc.gather_scatter(ref["rsT"], ref["ciT"], ref["rsT"], ref["ciT"], q)
    np.testing.assert_array_equal(host(dq), want)


@pytest.mark.parametrize("box", BOXES)
def test_box_gather_and_scatter_fp64(cuda, orc, box):
    nx, ny, nz, p, seed = box
    ids = O.box_hex_ids(nx, ny, nz, p, seed)
    h, ref = make(orc, ids)
    q = orc.uniform(ids.size, 23)
    ng = ref["rsT"].size - 1
    gq = torch.zeros(ng, dtype=torch.float64, device="cuda")
    h.Gather(gq, torch.from_numpy(q).cuda(), 1, O.Add, O.Trans)           # BS6
    np.testing.assert_array_equal(host(gq), orc.gather(ref["rsT"], ref["ciT"], q))
    g = orc.uniform(ng, 29)
    dq = torch.zeros(ids.size, dtype=torch.float64, device="cuda")
    h.Scatter(dq, torch.from_numpy(g).cuda(), 1, O.NoTrans)                # BS7
    np.testing.assert_array_equal(host(dq), orc.scatter(ref["rsT"], ref["ciT"], g,
                                                        np.zeros(ids.size)))


@pytest.mark.parametrize("kernel", [0, 1, 2, 3, 4, 5])
@pytest.mark.parametrize("box", [(2, 2, 2, 1), (2, 2, 2, 2), (3, 2, 2, 3), (2, 1, 1, 4)])
def test_small_plans_n_operator_every_kernel(cuda, orc, kernel, box):
    """Plans of one warp chunk, whose N operator has the same row range as T but
    fewer entries: every N-operator operation with every kernel variant."""
    saved = {key: capi.tune_get(key) for key in ("ogs.kernel", "ogs.kernel.gather",
                                                  "ogs.kernel.scatter")}
    try:
        capi.tune_set("ogs.kernel.gather", kernel)
        capi.tune_set("ogs.kernel.scatter", kernel)
        capi.tune_set("ogs.kernel", min(kernel, 3))
        ids = O.box_hex_ids(*box)
        h, ref = make(orc, ids)
        n, nT, nN = ids.size, ref["rsT"].size - 1, ref["rsN"].size - 1
        assert ref["ciN"].size < ref["ciT"].size
        q = orc.uniform(n, 41)
        gv = torch.zeros(max(nN, 1), dtype=torch.float64, device="cuda")
        h.Gather(gv, torch.from_numpy(q).cuda(), 1, O.Add, O.NoTrans)
        np.testing.assert_array_equal(host(gv)[:nN], orc.gather(ref["rsN"], ref["ciN"], q))
        g = orc.uniform(nT, 43)
        dv = torch.zeros(n, dtype=torch.float64, device="cuda")
        h.Scatter(dv, torch.from_numpy(g).cuda(), 1, O.Trans)
        np.testing.assert_array_equal(host(dv), orc.scatter(ref["rsN"], ref["ciN"], g[:nN],
                                                            np.zeros(n)))
        rsNp = pad(ref["rsN"], nT)
        for trans, (grs, gci, srs, sci) in ((O.NoTrans, (rsNp, ref["ciN"], ref["rsT"], ref["ciT"])),
                                            (O.Trans, (ref["rsT"], ref["ciT"], rsNp, ref["ciN"]))):
            dv = torch.from_numpy(q).cuda()
            h.GatherScatter(dv, 1, O.Add, trans)
            np.testing.assert_array_equal(host(dv), orc.gather_scatter(grs, gci, srs, sci, q),
                                          err_msg=f"gs trans={trans}")
    finally:
        for key, v in saved.items():
            capi.tune_set(key, v)


@pytest.mark.parametrize("tcode", [capi.FLOAT, capi.DOUBLE, capi.INT32, capi.INT64])
@pytest.mark.parametrize("op", [O.Add, O.Mul, O.Max, O.Min])
@pytest.mark.parametrize("k", [1, 3])
def test_all_types_ops_transposes(cuda, orc, tcode, op, k):
    rng = np.random.default_rng(1000 * tcode + 10 * op + k)
    n = 3000
    keys = rng.integers(1, 700, size=n).astype(np.int64)
    keys[rng.random(n) < 0.08] = 0            # ignored entries
    keys[rng.random(n) < 0.3] *= -1           # flagged entries
    h, ref = make(orc, keys, kind=capi.SIGNED, unique=False)
    nT, nN = ref["rsT"].size - 1, ref["rsN"].size - 1
    rsNp = pad(ref["rsN"], nT)
    dt = NP_TYPES[tcode]
    v = values(orc, n * k, dt, 5 + op)
    tv = torch.from_numpy(v).cuda()

    # Gather Trans / NoTrans
    for trans, (rs, ci, rows) in ((O.Trans, (ref["rsT"], ref["ciT"], nT)),
                                  (O.NoTrans, (ref["rsN"], ref["ciN"], nN))):
        gv = torch.zeros(max(rows, 1) * k, dtype=tv.dtype, device="cuda")
        h.Gather(gv, tv, k, op, trans)
        np.testing.assert_array_equal(host(gv)[: rows * k], orc.gather(rs, ci, v, k, op),
                                      err_msg=f"gather trans={trans}")
    # Scatter NoTrans (T) / Trans (N)
    for trans, (rs, ci, rows) in ((O.NoTrans, (ref["rsT"], ref["ciT"], nT)),
                                  (O.Trans, (ref["rsN"], ref["ciN"], nN))):
        g = values(orc, max(rows, 1) * k, dt, 77)
        base = values(orc, n * k, dt, 78)
        dv = torch.from_numpy(base).cuda()
        h.Scatter(dv, torch.from_numpy(g).cuda(), k, trans)
        np.testing.assert_array_equal(host(dv), orc.scatter(rs, ci, g[: rows * k], base, k),
                                      err_msg=f"scatter trans={trans}")
    # GatherScatter Sym / NoTrans / Trans (op honoured for every transpose)
    cases = {O.Sym: (ref["rsT"], ref["ciT"], ref["rsT"], ref["ciT"]),
             O.NoTrans: (rsNp, ref["ciN"], ref["rsT"], ref["ciT"]),
             O.Trans: (ref["rsT"], ref["ciT"], rsNp, ref["ciN"])}
    for trans, (grs, gci, srs, sci) in cases.items():
        dv = torch.from_numpy(v).cuda()
        h.GatherScatter(dv, k, op, trans)
        np.testing.assert_array_equal(host(dv), orc.gather_scatter(grs, gci, srs, sci, v, k, op),
                                      err_msg=f"gs trans={trans}")


def test_unsigned_handle(cuda, orc):
    rng = np.random.default_rng(5)
    n = 2000
    keys = rng.integers(1, 300, size=n).astype(np.int64)
    keys[rng.random(n) < 0.5] *= -1
    h, ref = make(orc, keys, kind=capi.UNSIGNED, unique=False)
    nN = ref["rsN"].size - 1
    v = orc.uniform(n, 3)
    tv = torch.from_numpy(v).cuda()
    gv = torch.zeros(nN, dtype=torch.float64, device="cuda")
    h.Gather(gv, tv, 1, O.Add, O.NoTrans)
    np.testing.assert_array_equal(host(gv), orc.gather(ref["rsN"], ref["ciN"], v))
    for trans in (O.Sym, O.NoTrans, O.Trans):
        dv = torch.from_numpy(v).cuda()
        h.GatherScatter(dv, 1, O.Add, trans)
        np.testing.assert_array_equal(
            host(dv), orc.gather_scatter(ref["rsT"], ref["ciT"], ref["rsT"], ref["ciT"], v))


def test_negative_zero_and_special_values(cuda, orc):
    # 0.0 + (-0.0) = +0.0 in the reference's row sums; NaN never wins Max/Min
    ids = np.array([1, 1, 2, 3, 3, 3], dtype=np.int64)
    h, ref = make(orc, ids)
    v = np.array([-0.0, -0.0, -0.0, np.nan, 1.0, -np.inf])
    for op in (O.Add, O.Max, O.Min, O.Mul):
        dv = torch.from_numpy(v).cuda()
        h.GatherScatter(dv, 1, op, O.Sym)
        want = orc.gather_scatter(ref["rsT"], ref["ciT"], ref["rsT"], ref["ciT"], v, 1, op)
        got = host(dv)
        np.testing.assert_array_equal(np.signbit(got), np.signbit(want))
        np.testing.assert_array_equal(got, want)


def test_empty_and_tiny_plans(cuda, orc):
    h = O.ogs_t()
    ids = np.zeros(5, dtype=np.int64)
    h.Setup(5, ids, unique=True)
    assert h.NgatherGlobal == 0
    v = torch.ones(5, dtype=torch.float64, device="cuda")
    h.GatherScatter(v, 1, O.Add, O.Sym)
    assert host(v).tolist() == [1.0] * 5
    ids = np.array([7], dtype=np.int64)
    h.Setup(1, ids, unique=True)
    v = torch.tensor([-0.0], dtype=torch.float64, device="cuda")
    h.GatherScatter(v, 1, O.Add, O.Sym)
    assert not np.signbit(host(v)[0])


def test_large_block_boundaries(cuda, orc):
    """Rows of varied multiplicity (up to the reference's 512 limit) crossing the
    2048-entry block boundaries."""
    rng = np.random.default_rng(11)
    sizes = rng.integers(1, 513, size=300)
    keys = np.repeat(np.arange(1, sizes.size + 1), sizes).astype(np.int64)
    rng.shuffle(keys)
    h, ref = make(orc, keys)
    v = orc.uniform(keys.size, 8)
    dv = torch.from_numpy(v).cuda()
    h.GatherScatter(dv, 1, O.Add, O.Sym)
    np.testing.assert_array_equal(
        host(dv), orc.gather_scatter(ref["rsT"], ref["ciT"], ref["rsT"], ref["ciT"], v))
    assert h.info.maxRowSize == sizes.max()


VARIANTS = [(0, 0, 0), (1, 0, 0), (1, 1, 1), (1, 2, 0), (2, 0, 0), (2, 1, 0), (2, 1, 1),
            (2, 2, 0), (2, 2, 1), (3, 0, 1), (3, 1, 0), (3, 1, 1), (3, 2, 1), (4, 0, 0),
            (4, 1, 0), (4, 1, 1), (4, 2, 1), (5, 0, 0), (5, 1, 1), (5, 2, 1)]
KNOBS = ("ogs.kernel", "ogs.kernel.gather", "ogs.kernel.scatter", "ogs.order", "ogs.rows")


def set_variant(kernel, order, rows):
    capi.tune_set("ogs.kernel", kernel)
    capi.tune_set("ogs.kernel.gather", kernel)
    capi.tune_set("ogs.kernel.scatter", kernel)
    capi.tune_set("ogs.order", order)
    capi.tune_set("ogs.rows", rows)


@pytest.mark.parametrize("kernel,order,rows", VARIANTS)
@pytest.mark.parametrize("box", [(5, 4, 3, 7, 2024), (6, 6, 6, 2, 5), (7, 3, 2, 1, 0)])
def test_kernel_variants_and_chunk_orders(cuda, orc, kernel, order, rows, box):
    """Block kernels, warp-chunk kernels (plain, pipelined, asynchronously staged
    gathers, column-order scatter and gathers, L2-prefetching gathers and scatter) in
    row order, breadth-first chunk order and the renumbered breadth-first walk, with
    rows in CSR order or grouped by size: all give the reference's bits (each row is
    still summed by one lane in CSR order)."""
    nx, ny, nz, p, seed = box
    old = {k: capi.tune_get(k) for k in KNOBS}
    try:
        set_variant(kernel, order, rows)
        ids = O.box_hex_ids(nx, ny, nz, p, seed)
        h, ref = make(orc, ids)
        assert h.info.chunkOrder == order and h.info.NchunksT > 0
        assert h.info.rowOrder == rows
        rs, ci = ref["rsT"], ref["ciT"]
        q = orc.uniform(ids.size, 91)
        gq = torch.zeros(rs.size - 1, dtype=torch.float64, device="cuda")
        h.Gather(gq, torch.from_numpy(q).cuda(), 1, O.Add, O.Trans)
        np.testing.assert_array_equal(host(gq), orc.gather(rs, ci, q))
        g = orc.uniform(rs.size - 1, 92)
        dq = torch.zeros(ids.size, dtype=torch.float64, device="cuda")
        h.Scatter(dq, torch.from_numpy(g).cuda(), 1, O.NoTrans)
        np.testing.assert_array_equal(host(dq), orc.scatter(rs, ci, g, np.zeros(ids.size)))
        dq = torch.from_numpy(q).cuda()
        h.GatherScatter(dq, 1, O.Add, O.Sym)
        np.testing.assert_array_equal(host(dq), orc.gather_scatter(rs, ci, rs, ci, q))
        gN = torch.zeros(ref["rsN"].size - 1, dtype=torch.float64, device="cuda")
        h.Gather(gN, torch.from_numpy(q).cuda(), 1, O.Add, O.NoTrans)
        np.testing.assert_array_equal(host(gN), orc.gather(ref["rsN"], ref["ciN"], q))
    finally:
        for k, v in old.items():
            capi.tune_set(k, v)


@pytest.mark.parametrize("kernel,rows", [(2, 1), (3, 0), (3, 1), (4, 0), (4, 1), (5, 1)])
@pytest.mark.parametrize("dtype", [torch.float32, torch.int32, torch.int64])
@pytest.mark.parametrize("op", [O.Add, O.Mul, O.Max, O.Min])
def test_variants_types_ops(cuda, orc, kernel, rows, dtype, op):
    """Every type and op through the warp-chunk variants with grouped rows, the
    asynchronously staged gathers (4- and 8-byte cp.async copies) and the
    column-order scatter and gathers."""
    old = {k: capi.tune_get(k) for k in KNOBS}
    try:
        set_variant(kernel, 1, rows)
        ids = O.box_hex_ids(4, 3, 5, 3, 77)
        h, ref = make(orc, ids)
        rs, ci = ref["rsT"], ref["ciT"]
        rng = np.random.default_rng(5)
        if dtype == torch.float32:
            q = rng.uniform(-1, 1, ids.size).astype(np.float32)
        else:
            q = rng.integers(-9, 10, ids.size).astype(np.int32 if dtype == torch.int32 else np.int64)
        gq = torch.zeros(rs.size - 1, dtype=dtype, device="cuda")
        h.Gather(gq, torch.from_numpy(q).cuda(), 1, op, O.Trans)
        np.testing.assert_array_equal(host(gq), orc.gather(rs, ci, q, 1, op))
        dq = torch.from_numpy(q.copy()).cuda()
        h.GatherScatter(dq, 1, op, O.Sym)
        np.testing.assert_array_equal(host(dq), orc.gather_scatter(rs, ci, rs, ci, q, 1, op))
        g = orc.gather(rs, ci, q, 1, op)
        dq = torch.zeros(ids.size, dtype=dtype, device="cuda")
        h.Scatter(dq, torch.from_numpy(g).cuda(), 1, O.NoTrans)
        np.testing.assert_array_equal(host(dq), orc.scatter(rs, ci, g, np.zeros_like(q)))
    finally:
        for k, v in old.items():
            capi.tune_set(k, v)


@pytest.mark.parametrize("knobs", [
    {"ogs.order": 1, "ogs.ball_shift": 12},
    {"ogs.order": 2, "ogs.page_shift": 6, "ogs.ball_shift": 10},
    {"ogs.order": 1, "ogs.gs_order": 2, "ogs.gs_page_shift": 8, "ogs.gs_ball_shift": 0},
    {"ogs.order": 0, "ogs.gs_order": 2, "ogs.gs_page_shift": 5, "ogs.gs_ball_shift": 11},
    {"ogs.order": 2, "ogs.rows": 0, "ogs.gs_order": 1, "ogs.gs_page_shift": 6,
     "ogs.gs_ball_shift": 14},
    {"ogs.order": 1, "ogs.rows": 0, "ogs.gs_order": 2, "ogs.gs_page_shift": 4,
     "ogs.gs_ball_shift": 0, "ogs.kernel": 5},
    {"ogs.order": 1, "ogs.gs_order": 0, "ogs.kernel": 1}])
@pytest.mark.parametrize("box", [(5, 4, 3, 7, 2024), (6, 6, 6, 2, 5)])
def test_ball_chains_and_gather_scatter_walks(cuda, orc, knobs, box):
    """Chains of balls for the main walk, and a second walk for the in-place
    gather+scatter: every operation stays bit-exact."""
    names = ["ogs.order", "ogs.rows", "ogs.page_shift", "ogs.ball_shift", "ogs.gs_order",
             "ogs.gs_page_shift", "ogs.gs_ball_shift", "ogs.kernel"]
    saved = {n: capi.tune_get(n) for n in names}
    try:
        for n, v in knobs.items():
            capi.tune_set(n, v)
        nx, ny, nz, p, seed = box
        ids = O.box_hex_ids(nx, ny, nz, p, seed)
        h, ref = make(orc, ids)
        gs_walk = knobs.get("ogs.gs_order", -1) >= 0
        assert (h.info.NchunksGS > 0) == gs_walk
        if gs_walk:
            assert h.info.gsRowOrder == capi.tune_get("ogs.rows")
        q = orc.uniform(ids.size, 61)
        for op in (O.Add, O.Max):
            dq = torch.from_numpy(q).cuda()
            h.GatherScatter(dq, 1, op, O.Sym)
            np.testing.assert_array_equal(
                host(dq), orc.gather_scatter(ref["rsT"], ref["ciT"], ref["rsT"], ref["ciT"], q, 1,
                                             op), err_msg=f"gs op={op}")
        ng = ref["rsT"].size - 1
        gq = torch.zeros(ng, dtype=torch.float64, device="cuda")
        h.Gather(gq, torch.from_numpy(q).cuda(), 1, O.Add, O.Trans)
        np.testing.assert_array_equal(host(gq), orc.gather(ref["rsT"], ref["ciT"], q))
        nT = ng
        rsNp = pad(ref["rsN"], nT)
        dq = torch.from_numpy(q).cuda()
        h.GatherScatter(dq, 1, O.Add, O.NoTrans)
        np.testing.assert_array_equal(
            host(dq), orc.gather_scatter(rsNp, ref["ciN"], ref["rsT"], ref["ciT"], q))
    finally:
        for n, v in saved.items():
            capi.tune_set(n, v)


@pytest.mark.parametrize("shift", [3, 6, 12])
@pytest.mark.parametrize("order", [1, 2])
def test_page_sizes_of_breadth_first_order(cuda, orc, shift, order):
    """Breadth-first chunk order, and the renumbered breadth-first walk, over pages
    of 8, 64 and 4096 entries: the same bits."""
    old = {k: capi.tune_get(k) for k in KNOBS + ("ogs.page_shift",)}
    try:
        set_variant(2, order, 1)
        capi.tune_set("ogs.page_shift", shift)
        ids = O.box_hex_ids(5, 4, 6, 3, 31)
        h, ref = make(orc, ids)
        assert h.info.chunkOrder == order and h.info.NchunksT > 0
        rs, ci = ref["rsT"], ref["ciT"]
        q = orc.uniform(ids.size, 5)
        gq = torch.zeros(rs.size - 1, dtype=torch.float64, device="cuda")
        h.Gather(gq, torch.from_numpy(q).cuda(), 1, O.Add, O.Trans)
        np.testing.assert_array_equal(host(gq), orc.gather(rs, ci, q))
        dq = torch.from_numpy(q).cuda()
        h.GatherScatter(dq, 1, O.Add, O.Sym)
        np.testing.assert_array_equal(host(dq), orc.gather_scatter(rs, ci, rs, ci, q))
        g = orc.uniform(rs.size - 1, 6)
        dq = torch.zeros(ids.size, dtype=torch.float64, device="cuda")
        h.Scatter(dq, torch.from_numpy(g).cuda(), 1, O.NoTrans)
        np.testing.assert_array_equal(host(dq), orc.scatter(rs, ci, g, np.zeros(ids.size)))
    finally:
        for k, v in old.items():
            capi.tune_set(k, v)


@pytest.mark.parametrize("n", [1, 2, 3, 5, 7, 81, 405, 1001, 4099])
@pytest.mark.parametrize("dtype", [np.float32, np.float64, np.int32, np.int64])
@pytest.mark.parametrize("offset", [0, 1])
@pytest.mark.parametrize("walk", [(0, 9, 1), (1, 8, 0), (1, 8, 1), (2, 8, 1), (1, 9, 1), (1, 3, 1)])
def test_column_major_scatter_any_length(cuda, orc, n, dtype, offset, walk):
    """The column-major scatter with 16-byte accesses (kernel 5) for every length
    modulo the vector width, in memory order and with its pages in the walk's order
    (chunk order, page shift, ogs.scatter_pages), with columns in no row (id 0)
    keeping their values and the vector shifted off its 16-byte alignment (the
    one-column form then runs)."""
    keys = ("ogs.kernel.scatter", "ogs.order", "ogs.page_shift", "ogs.scatter_pages")
    old = {k: capi.tune_get(k) for k in keys}
    try:
        for k, x in zip(keys, (5,) + walk):
            capi.tune_set(k, x)
        rng = np.random.default_rng(n * 7 + offset)
        ids = rng.integers(-max(2, n // 3), max(2, n // 3) + 1, n).astype(np.int64)
        ids[0] = ids[0] or 1
        h, ref = make(orc, ids)
        assert h.info.NpagesT == (0 if walk[0] == 0 else -(-n // (1 << walk[1])))
        assert h.info.NpagesT == 0 or h.info.pageShift == walk[1]
        rs, ci = ref["rsT"], ref["ciT"]
        g = values(orc, rs.size - 1, dtype, 17)
        base = values(orc, n, dtype, 19)
        store = torch.from_numpy(np.concatenate([np.zeros(offset, dtype), base])).cuda()
        dq = store[offset:]
        h.Scatter(dq, torch.from_numpy(g).cuda(), 1, O.NoTrans)
        np.testing.assert_array_equal(host(dq), orc.scatter(rs, ci, g, base))
    finally:
        for k, x in old.items():
            capi.tune_set(k, x)


BULK_KNOBS = ("ogs.kernel", "ogs.kernel.gather", "ogs.order", "ogs.rows", "ogs.gs_order",
              "ogs.page_shift", "ogs.ball_shift")


@pytest.mark.parametrize("knobs", [
    {"ogs.order": 0}, {"ogs.order": 1}, {"ogs.order": 2, "ogs.page_shift": 6},
    {"ogs.order": 1, "ogs.ball_shift": 12, "ogs.gs_order": 2},
    {"ogs.order": 1, "ogs.rows": 0, "ogs.gs_order": 1}])
@pytest.mark.parametrize("box", [(5, 4, 3, 7, 2024), (6, 6, 6, 2, 5), (7, 3, 2, 1, 0),
                                 (3, 3, 3, 15, 4), (1, 1, 1, 1, 0)])
def test_bulk_staged_gathers(cuda, orc, knobs, box):
    """Kernel 6 (the pipelined gathers with each chunk's column ids brought to shared
    memory by TMA bulk copy, one chunk ahead) for the gather, the gather through the
    N operator and the gather+scatter with every op, on every walk: the reference's
    bits, and no bounded staging wait gave up."""
    saved = {n: capi.tune_get(n) for n in BULK_KNOBS}
    try:
        capi.tune_set("ogs.kernel", 6)
        capi.tune_set("ogs.kernel.gather", 6)
        for n, v in knobs.items():
            capi.tune_set(n, v)
        nx, ny, nz, p, seed = box
        ids = O.box_hex_ids(nx, ny, nz, p, seed)
        h, ref = make(orc, ids)
        rs, ci = ref["rsT"], ref["ciT"]
        q = orc.uniform(ids.size, 71)
        gq = torch.zeros(rs.size - 1, dtype=torch.float64, device="cuda")
        h.Gather(gq, torch.from_numpy(q).cuda(), 1, O.Add, O.Trans)
        np.testing.assert_array_equal(host(gq), orc.gather(rs, ci, q))
        gN = torch.zeros(ref["rsN"].size - 1, dtype=torch.float64, device="cuda")
        h.Gather(gN, torch.from_numpy(q).cuda(), 1, O.Add, O.NoTrans)
        np.testing.assert_array_equal(host(gN), orc.gather(ref["rsN"], ref["ciN"], q))
        for op in (O.Add, O.Mul, O.Max, O.Min):
            dq = torch.from_numpy(q).cuda()
            h.GatherScatter(dq, 1, op, O.Sym)
            np.testing.assert_array_equal(host(dq), orc.gather_scatter(rs, ci, rs, ci, q, 1, op),
                                          err_msg=f"op {op}")
        assert h.plan_info().waitErrors == 0
    finally:
        for n, v in saved.items():
            capi.tune_set(n, v)


@pytest.mark.parametrize("dtype", [torch.float32, torch.int32, torch.int64])
@pytest.mark.parametrize("op", [O.Add, O.Mul, O.Max, O.Min])
def test_bulk_staged_gathers_types(cuda, orc, dtype, op):
    saved = {n: capi.tune_get(n) for n in BULK_KNOBS}
    try:
        capi.tune_set("ogs.kernel", 6)
        capi.tune_set("ogs.kernel.gather", 6)
        ids = O.box_hex_ids(4, 3, 5, 3, 77)
        h, ref = make(orc, ids)
        rs, ci = ref["rsT"], ref["ciT"]
        rng = np.random.default_rng(6)
        if dtype == torch.float32:
            q = rng.uniform(-1, 1, ids.size).astype(np.float32)
            q[::37] = -0.0
        else:
            q = rng.integers(-9, 10, ids.size).astype(np.int32 if dtype == torch.int32 else np.int64)
        gq = torch.zeros(rs.size - 1, dtype=dtype, device="cuda")
        h.Gather(gq, torch.from_numpy(q).cuda(), 1, op, O.Trans)
        np.testing.assert_array_equal(host(gq), orc.gather(rs, ci, q, 1, op))
        dq = torch.from_numpy(q.copy()).cuda()
        h.GatherScatter(dq, 1, op, O.Sym)
        np.testing.assert_array_equal(host(dq), orc.gather_scatter(rs, ci, rs, ci, q, 1, op))
        assert h.plan_info().waitErrors == 0
    finally:
        for n, v in saved.items():
            capi.tune_set(n, v)


def test_bulk_staged_gathers_large_groups(cuda, orc):
    """Random ids with groups of up to ~20 members, chunks starting at every offset
    modulo 4 (the bulk copy's 16-byte aligned span around each chunk's ids)."""
    saved = {n: capi.tune_get(n) for n in BULK_KNOBS}
    try:
        capi.tune_set("ogs.kernel", 6)
        capi.tune_set("ogs.kernel.gather", 6)
        rng = np.random.default_rng(3)
        ids = rng.integers(1, 600, 5003).astype(np.int64)
        h, ref = make(orc, ids)
        rs, ci = ref["rsT"], ref["ciT"]
        q = orc.uniform(ids.size, 5)
        dq = torch.from_numpy(q).cuda()
        h.GatherScatter(dq, 1, O.Add, O.Sym)
        np.testing.assert_array_equal(host(dq), orc.gather_scatter(rs, ci, rs, ci, q))
        gq = torch.zeros(rs.size - 1, dtype=torch.float64, device="cuda")
        h.Gather(gq, torch.from_numpy(q).cuda(), 1, O.Add, O.Trans)
        np.testing.assert_array_equal(host(gq), orc.gather(rs, ci, q))
        assert h.plan_info().waitErrors == 0
    finally:
        for n, v in saved.items():
            capi.tune_set(n, v)


SINGLE_KNOBS = ("ogs.kernel", "ogs.kernel.gather", "ogs.order", "ogs.rows", "ogs.gs_order",
                "ogs.page_shift", "ogs.ball_shift", "ogs.singles")


@pytest.mark.parametrize("knobs", [
    {"ogs.order": 0}, {"ogs.order": 1}, {"ogs.order": 2, "ogs.page_shift": 6},
    {"ogs.order": 1, "ogs.ball_shift": 12, "ogs.gs_order": 2},
    {"ogs.order": 1, "ogs.gs_order": 1, "ogs.gs_page_shift": 6}])
@pytest.mark.parametrize("box", [(5, 4, 3, 7, 2024), (6, 6, 6, 2, 5), (7, 3, 2, 1, 0),
                                 (3, 3, 3, 15, 4)])
@pytest.mark.parametrize("singles", [1, 2])
def test_single_member_rows_path(cuda, orc, knobs, box, singles):
    """Kernel 2 with ogs.singles = 1: rows of one member bypass the staging; the
    gather, the N-operator gather and the gather+scatter keep the reference's bits
    for every op, including values whose first step changes them (-0 under Add,
    -Inf and NaN under Max and Min)."""
    saved = {n: capi.tune_get(n) for n in SINGLE_KNOBS + ("ogs.gs_page_shift",)}
    try:
        capi.tune_set("ogs.kernel", 2)
        capi.tune_set("ogs.kernel.gather", 2)
        capi.tune_set("ogs.rows", 1)
        capi.tune_set("ogs.singles", singles)
        for n, v in knobs.items():
            capi.tune_set(n, v)
        nx, ny, nz, p, seed = box
        ids = O.box_hex_ids(nx, ny, nz, p, seed)
        h, ref = make(orc, ids)
        rs, ci = ref["rsT"], ref["ciT"]
        q = orc.uniform(ids.size, 81)
        q[::11] = -0.0
        q[::53] = -np.inf
        q[::59] = np.nan
        q[::61] = np.inf
        gq = torch.zeros(rs.size - 1, dtype=torch.float64, device="cuda")
        for op in (O.Add, O.Max, O.Min):
            # equal values (NaN where the oracle has NaN) and equal signs of zeros
            h.Gather(gq, torch.from_numpy(q).cuda(), 1, op, O.Trans)
            got, want = host(gq), orc.gather(rs, ci, q, 1, op)
            np.testing.assert_array_equal(got, want)
            ok = ~np.isnan(want)  # a NaN made from Inf - Inf has no portable sign
            np.testing.assert_array_equal(np.signbit(got[ok]), np.signbit(want[ok]))
            dq = torch.from_numpy(q).cuda()
            h.GatherScatter(dq, 1, op, O.Sym)
            got, want = host(dq), orc.gather_scatter(rs, ci, rs, ci, q, 1, op)
            np.testing.assert_array_equal(got, want, err_msg=f"op {op}")
            ok = ~np.isnan(want)
            np.testing.assert_array_equal(np.signbit(got[ok]), np.signbit(want[ok]))
        qf = orc.uniform(ids.size, 82)
        gN = torch.zeros(ref["rsN"].size - 1, dtype=torch.float64, device="cuda")
        h.Gather(gN, torch.from_numpy(qf).cuda(), 1, O.Add, O.NoTrans)
        np.testing.assert_array_equal(host(gN), orc.gather(ref["rsN"], ref["ciN"], qf))
    finally:
        for n, v in saved.items():
            capi.tune_set(n, v)


@pytest.mark.parametrize("dtype", [torch.float32, torch.int32, torch.int64])
@pytest.mark.parametrize("op", [O.Add, O.Mul, O.Max, O.Min])
@pytest.mark.parametrize("singles", [1, 2])
def test_single_member_rows_path_types(cuda, orc, dtype, op, singles):
    saved = {n: capi.tune_get(n) for n in SINGLE_KNOBS}
    try:
        capi.tune_set("ogs.kernel", 2)
        capi.tune_set("ogs.kernel.gather", 2)
        capi.tune_set("ogs.rows", 1)
        capi.tune_set("ogs.singles", singles)
        ids = O.box_hex_ids(4, 3, 5, 3, 77)
        h, ref = make(orc, ids)
        rs, ci = ref["rsT"], ref["ciT"]
        rng = np.random.default_rng(9)
        if dtype == torch.float32:
            q = rng.uniform(-1, 1, ids.size).astype(np.float32)
            q[::37] = -0.0
            q[::41] = -np.inf
        else:
            q = rng.integers(-9, 10, ids.size).astype(np.int32 if dtype == torch.int32 else np.int64)
        gq = torch.zeros(rs.size - 1, dtype=dtype, device="cuda")
        h.Gather(gq, torch.from_numpy(q).cuda(), 1, op, O.Trans)
        np.testing.assert_array_equal(host(gq), orc.gather(rs, ci, q, 1, op))
        dq = torch.from_numpy(q.copy()).cuda()
        h.GatherScatter(dq, 1, op, O.Sym)
        np.testing.assert_array_equal(host(dq), orc.gather_scatter(rs, ci, rs, ci, q, 1, op))
    finally:
        for n, v in saved.items():
            capi.tune_set(n, v)
