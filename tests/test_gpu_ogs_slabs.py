"""Lane-row slab gathers (kernel 7) against the oracle's host loops (GPU).

Kernel 7 combines every row in registers of one lane, rows of equal size side by
side, from the slab layout the plan builds (rows regrouped by size inside segments
of the walk, member-major ids).  Each row is still summed from the op's first step
in its CSR order, so every type, op and layout gives the reference's bits
(ogsOperator.cpp:382-385, ogsKernels.okl:64-67)."""
import numpy as np
import pytest
import torch

from streamparanumal_gb300 import capi
from streamparanumal_gb300 import ogs as O

pytestmark = pytest.mark.gpu

KNOBS = ("ogs.kernel", "ogs.kernel.gather", "ogs.order", "ogs.rows", "ogs.gs_order",
         "ogs.gs_page_shift", "ogs.gs_ball_shift", "ogs.slabs", "ogs.slab_seg_shift",
         "ogs.slab_lane", "ogs.slab_ctas", "ogs.slab_load", "ogs.slab_defer",
         "ogs.slab_code_shift", "ogs.kernel.f32", "ogs.kernel.gather.f32", "ogs.page_shift",
         "ogs.ball_shift", "ogs.slab_row_codes")


@pytest.fixture
def knobs():
    saved = {k: capi.tune_get(k) for k in KNOBS}
    capi.tune_set("ogs.kernel", 7)
    capi.tune_set("ogs.kernel.gather", 7)
    capi.tune_set("ogs.slabs", 1)
    yield capi.tune_set
    for k, v in saved.items():
        capi.tune_set(k, v)


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def make(orc, ids, kind=capi.SIGNED, unique=True):
    ref = orc.ogs_setup(ids.copy(), kind=kind, unique=unique)
    h = O.ogs_t()
    h.Setup(ids.size, ids.copy(), kind=kind, unique=unique)
    return h, ref


def check_fp64(orc, h, ref, n, seed):
    rs, ci = ref["rsT"], ref["ciT"]
    q = orc.uniform(n, seed)
    gq = torch.zeros(rs.size - 1, dtype=torch.float64, device="cuda")
    h.Gather(gq, torch.from_numpy(q).cuda(), 1, O.Add, O.Trans)                 # BS6
    np.testing.assert_array_equal(host(gq), orc.gather(rs, ci, q))
    dq = torch.from_numpy(q).cuda()
    h.GatherScatter(dq, 1, O.Add, O.Sym)                                        # BS8
    np.testing.assert_array_equal(host(dq), orc.gather_scatter(rs, ci, rs, ci, q))
    gN = torch.zeros(ref["rsN"].size - 1, dtype=torch.float64, device="cuda")
    h.Gather(gN, torch.from_numpy(q).cuda(), 1, O.Add, O.NoTrans)              # N: kernel 2
    np.testing.assert_array_equal(host(gN), orc.gather(ref["rsN"], ref["ciN"], q))


BOXES = [(2, 2, 2, 1, 0), (5, 4, 3, 7, 2024), (6, 6, 6, 2, 5), (7, 3, 2, 1, 0), (4, 3, 5, 3, 77),
         (9, 8, 7, 5, 3), (16, 16, 16, 7, 0)]


@pytest.mark.parametrize("box", BOXES)
@pytest.mark.parametrize("order,rows,gs_order", [(0, 1, -1), (1, 1, -1), (2, 1, -1), (1, 0, 2),
                                                 (2, 1, 2), (1, 1, 0)])
def test_slabs_fp64_every_walk(cuda, orc, knobs, box, order, rows, gs_order):
    nx, ny, nz, p, seed = box
    knobs("ogs.order", order)
    knobs("ogs.rows", rows)
    knobs("ogs.gs_order", gs_order)
    knobs("ogs.gs_page_shift", 6)
    knobs("ogs.gs_ball_shift", 0)
    ids = O.box_hex_ids(nx, ny, nz, p, seed)
    h, ref = make(orc, ids)
    assert h.info.NslabsT > 0
    assert (h.info.NslabsGS > 0) == (h.info.NchunksGS > 0)
    check_fp64(orc, h, ref, ids.size, 31 + p)


@pytest.mark.parametrize("seg", [8, 10, 22])
@pytest.mark.parametrize("lane", [0, 8, 16])
@pytest.mark.parametrize("shift", [0, 8])
def test_slab_segments_and_kernel_shapes(cuda, orc, knobs, seg, lane, shift):
    """Small segments leave many partial slabs (their last row step partly filled,
    steps of fewer than 32 lanes) between full passes; 8 or 16 members in flight
    per lane, for FP64 and FP32, with 32-bit words or member and row codes, give
    the same bits."""
    knobs("ogs.slab_seg_shift", seg)
    knobs("ogs.slab_lane", lane)
    knobs("ogs.slab_code_shift", shift)
    knobs("ogs.slab_row_codes", 1)
    knobs("ogs.order", 1)
    ids = O.box_hex_ids(6, 5, 4, 5, 2024)
    h, ref = make(orc, ids)
    assert (h.info.slabCodedRows > 0) == (shift > 0)
    check_fp64(orc, h, ref, ids.size, 7)
    rs, ci = ref["rsT"], ref["ciT"]
    q = orc.uniform(ids.size, 8).astype(np.float32)
    gq = torch.zeros(rs.size - 1, dtype=torch.float32, device="cuda")
    h.Gather(gq, torch.from_numpy(q).cuda(), 1, O.Add, O.Trans)
    np.testing.assert_array_equal(host(gq), orc.gather(rs, ci, q))
    dq = torch.from_numpy(q.copy()).cuda()
    h.GatherScatter(dq, 1, O.Add, O.Sym)
    np.testing.assert_array_equal(host(dq), orc.gather_scatter(rs, ci, rs, ci, q))


@pytest.mark.parametrize("load", [1, 2, 3])
@pytest.mark.parametrize("ctas", [1, 3, 4])
@pytest.mark.parametrize("shift", [0, 9])
def test_slab_load_paths_and_ctas(cuda, orc, knobs, load, ctas, shift):
    """The value-load variants (L2 only, evict-first, read-only path) and the
    resident-CTA shapes of kernel 7 (with 32-bit words or member and row codes)
    give the same bits, FP64 and FP32."""
    knobs("ogs.order", 1)
    knobs("ogs.slab_code_shift", shift)
    knobs("ogs.slab_row_codes", 1)
    knobs("ogs.slab_load", load)
    ids = O.box_hex_ids(6, 5, 4, 7, 2024)
    h, ref = make(orc, ids)
    check_fp64(orc, h, ref, ids.size, 5)
    knobs("ogs.slab_load", 0)
    knobs("ogs.slab_ctas", ctas)
    check_fp64(orc, h, ref, ids.size, 6)
    rs, ci = ref["rsT"], ref["ciT"]
    for lv in (load, 0):
        knobs("ogs.slab_load", lv)
        q = orc.uniform(ids.size, 10 + lv).astype(np.float32)
        gq = torch.zeros(rs.size - 1, dtype=torch.float32, device="cuda")
        h.Gather(gq, torch.from_numpy(q).cuda(), 1, O.Add, O.Trans)
        np.testing.assert_array_equal(host(gq), orc.gather(rs, ci, q))
        dq = torch.from_numpy(q.copy()).cuda()
        h.GatherScatter(dq, 1, O.Add, O.Sym)
        np.testing.assert_array_equal(host(dq), orc.gather_scatter(rs, ci, rs, ci, q))


@pytest.mark.parametrize("seg", [8, 17])
@pytest.mark.parametrize("lane", [0, 16])
def test_slab_deferred_stores(cuda, orc, knobs, seg, lane):
    """The gather+scatter with each pass's stores issued after the next pass's
    loads (ogs.slab_defer): the same bits, FP64 and FP32, with -0 made +0."""
    knobs("ogs.order", 1)
    knobs("ogs.slab_seg_shift", seg)
    knobs("ogs.slab_lane", lane)
    knobs("ogs.slab_defer", 1)
    ids = O.box_hex_ids(7, 5, 4, 5, 31)
    h, ref = make(orc, ids)
    rs, ci = ref["rsT"], ref["ciT"]
    for dt in (np.float64, np.float32):
        q = orc.uniform(ids.size, 40).astype(dt)
        q[::7] = -0.0
        dq = torch.from_numpy(q.copy()).cuda()
        h.GatherScatter(dq, 1, O.Add, O.Sym)
        want = orc.gather_scatter(rs, ci, rs, ci, q)
        got = host(dq)
        np.testing.assert_array_equal(got, want)
        np.testing.assert_array_equal(np.signbit(got), np.signbit(want))


@pytest.mark.parametrize("box,shift", [((5, 4, 3, 7, 2024), 9), ((6, 6, 6, 2, 5), 5),
                                       ((9, 8, 7, 5, 3), 8), ((7, 3, 2, 1, 0), 3),
                                       ((4, 3, 5, 3, 77), 12), ((16, 16, 16, 7, 0), 6)])
@pytest.mark.parametrize("order,gs_order", [(1, -1), (2, 2)])
def test_slabs_with_16bit_codes(cuda, orc, knobs, box, shift, order, gs_order):
    """Slabs whose ids fit 16-bit codes (ogs.slab_code_shift) decode them through the
    slab's table in shared memory; the others keep 32-bit ids: the same bits for
    the gather and the gather+scatter, FP64 and FP32, with the deferred stores too."""
    nx, ny, nz, p, seed = box
    knobs("ogs.order", order)
    knobs("ogs.gs_order", gs_order)
    knobs("ogs.gs_page_shift", 6)
    knobs("ogs.gs_ball_shift", 0)
    knobs("ogs.slab_code_shift", shift)
    ids = O.box_hex_ids(nx, ny, nz, p, seed)
    h, ref = make(orc, ids)
    assert h.info.slabCodeShift == shift and h.info.slabCodedEntries > 0
    assert h.info.slabCodedRows == 0  # row codes are opt-in (ogs.slab_row_codes)
    check_fp64(orc, h, ref, ids.size, 11 + p)
    rs, ci = ref["rsT"], ref["ciT"]
    q = orc.uniform(ids.size, 12).astype(np.float32)
    gq = torch.zeros(rs.size - 1, dtype=torch.float32, device="cuda")
    h.Gather(gq, torch.from_numpy(q).cuda(), 1, O.Add, O.Trans)
    np.testing.assert_array_equal(host(gq), orc.gather(rs, ci, q))
    for defer in (0, 1):
        knobs("ogs.slab_defer", defer)
        dq = torch.from_numpy(q.copy()).cuda()
        h.GatherScatter(dq, 1, O.Add, O.Sym)
        np.testing.assert_array_equal(host(dq), orc.gather_scatter(rs, ci, rs, ci, q))


@pytest.mark.parametrize("box,shift", [((5, 4, 3, 7, 2024), 9), ((7, 3, 2, 1, 0), 3),
                                       ((4, 3, 5, 3, 77), 12), ((9, 8, 7, 5, 3), 8),
                                       ((16, 16, 16, 7, 0), 6)])
@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("lane", [0, 16])
def test_slab_row_codes(cuda, orc, knobs, box, shift, order, lane):
    """The gather's row words as 16-bit codes (ogs.slab_row_codes, with member
    codes): kernel 7's default Add gather decodes them through each slab's row
    table, the other shapes and ops read the 32-bit words the plan keeps -- the
    oracle's bits for every type and op either way (a slab of more than 32 row
    runs, or one whose codes do not fit 16 bits, keeps its words; order 2 renumbers
    the walk, so its rows are the plan's permuted row words)."""
    nx, ny, nz, p, seed = box
    knobs("ogs.order", order)
    knobs("ogs.slab_lane", lane)
    knobs("ogs.slab_code_shift", shift)
    ids = O.box_hex_ids(nx, ny, nz, p, seed)
    rng = np.random.default_rng(p)
    for rc in (1, 0):
        knobs("ogs.slab_row_codes", rc)
        h, ref = make(orc, ids)
        assert (h.info.slabCodedRows > 0) == bool(rc)
        assert h.info.slabCodedRows <= h.info.NrowsT
        rs, ci = ref["rsT"], ref["ciT"]
        for dt, tdt in ((np.float64, torch.float64), (np.float32, torch.float32),
                        (np.int32, torch.int32), (np.int64, torch.int64)):
            if dt in (np.float64, np.float32):
                q = rng.uniform(-1, 1, ids.size).astype(dt)
            else:
                q = rng.integers(-9, 10, ids.size).astype(dt)
            for op in (O.Add, O.Mul, O.Max, O.Min):
                gq = torch.zeros(rs.size - 1, dtype=tdt, device="cuda")
                h.Gather(gq, torch.from_numpy(q).cuda(), 1, op, O.Trans)
                np.testing.assert_array_equal(host(gq), orc.gather(rs, ci, q, 1, op))


@pytest.mark.parametrize("k64,k32", [(2, 7), (7, 2), (7, -1)])
def test_4byte_values_take_their_own_kernel(cuda, orc, knobs, k64, k32):
    """ogs.kernel.f32 / ogs.kernel.gather.f32 pick the kernels of 4-byte values
    apart from 8-byte ones; the bits do not change."""
    knobs("ogs.order", 1)
    knobs("ogs.slab_code_shift", 9)
    ids = O.box_hex_ids(5, 4, 3, 7, 2024)
    h, ref = make(orc, ids)
    for key in ("ogs.kernel", "ogs.kernel.gather"):
        knobs(key, k64)
    for key in ("ogs.kernel.f32", "ogs.kernel.gather.f32"):
        knobs(key, k32)
    check_fp64(orc, h, ref, ids.size, 21)
    rs, ci = ref["rsT"], ref["ciT"]
    for dt, tdt in ((np.float32, torch.float32), (np.int32, torch.int32)):
        q = orc.uniform(ids.size, 22).astype(np.float32)
        q = q if dt == np.float32 else np.round(q * 1000).astype(np.int32)
        gq = torch.zeros(rs.size - 1, dtype=tdt, device="cuda")
        h.Gather(gq, torch.from_numpy(q).cuda(), 1, O.Add, O.Trans)
        np.testing.assert_array_equal(host(gq), orc.gather(rs, ci, q))
        dq = torch.from_numpy(q.copy()).cuda()
        h.GatherScatter(dq, 1, O.Add, O.Sym)
        np.testing.assert_array_equal(host(dq), orc.gather_scatter(rs, ci, rs, ci, q))


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64, torch.int32, torch.int64])
@pytest.mark.parametrize("op", [O.Add, O.Mul, O.Max, O.Min])
@pytest.mark.parametrize("lane", [0, 16])
def test_slabs_types_ops(cuda, orc, knobs, dtype, op, lane):
    knobs("ogs.order", 1)
    knobs("ogs.slab_lane", lane)
    knobs("ogs.slab_code_shift", 6 if lane else 0)
    ids = O.box_hex_ids(4, 3, 5, 3, 77)
    h, ref = make(orc, ids)
    rs, ci = ref["rsT"], ref["ciT"]
    rng = np.random.default_rng(5)
    if dtype in (torch.float32, torch.float64):
        q = rng.uniform(-1, 1, ids.size).astype(np.float32 if dtype == torch.float32
                                                 else np.float64)
    else:
        q = rng.integers(-9, 10, ids.size).astype(np.int32 if dtype == torch.int32 else np.int64)
    gq = torch.zeros(rs.size - 1, dtype=dtype, device="cuda")
    h.Gather(gq, torch.from_numpy(q).cuda(), 1, op, O.Trans)
    np.testing.assert_array_equal(host(gq), orc.gather(rs, ci, q, 1, op))
    dq = torch.from_numpy(q.copy()).cuda()
    h.GatherScatter(dq, 1, op, O.Sym)
    np.testing.assert_array_equal(host(dq), orc.gather_scatter(rs, ci, rs, ci, q, 1, op))


@pytest.mark.parametrize("seg", [8, 14])
def test_slabs_any_row_size(cuda, orc, knobs, seg):
    """Groups of 1 to 40 members (sizes other than 1, 2, 4, 8 take the general row
    path; more than 16 members run in batches) with ignored and flagged entries."""
    knobs("ogs.slab_seg_shift", seg)
    knobs("ogs.order", 1)
    rng = np.random.default_rng(12)
    sizes = rng.integers(1, 41, size=700)
    keys = np.repeat(np.arange(1, sizes.size + 1), sizes).astype(np.int64)
    rng.shuffle(keys)
    keys[rng.random(keys.size) < 0.05] = 0
    keys[rng.random(keys.size) < 0.2] *= -1
    h, ref = make(orc, keys, unique=False)
    assert h.info.maxRowSize > 16
    for dtype in (np.float64, np.float32):
        q = orc.uniform(keys.size, 3).astype(dtype)
        rs, ci = ref["rsT"], ref["ciT"]
        gq = torch.zeros(rs.size - 1, dtype=torch.from_numpy(q).dtype, device="cuda")
        h.Gather(gq, torch.from_numpy(q).cuda(), 1, O.Add, O.Trans)
        np.testing.assert_array_equal(host(gq), orc.gather(rs, ci, q))
        dq = torch.from_numpy(q.copy()).cuda()
        h.GatherScatter(dq, 1, O.Max, O.Sym)
        np.testing.assert_array_equal(host(dq), orc.gather_scatter(rs, ci, rs, ci, q, 1, O.Max))


def test_slabs_rows_without_members(cuda, orc, knobs):
    """An explicit T operator with empty rows: the gather writes the op's identity
    there (rows of 0 members are slabs of their own)."""
    rng = np.random.default_rng(4)
    sizes = rng.integers(0, 10, size=2500)
    n = int(sizes.sum())
    rs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int32)
    ci = rng.permutation(n).astype(np.int32)
    h = O.ogs_t()
    h.SetupFromCSR(n, rs, ci)
    assert h.info.NslabsT > 0
    q = orc.uniform(n, 9)
    for op in (O.Add, O.Mul, O.Max, O.Min):
        gq = torch.full((rs.size - 1,), 5.0, dtype=torch.float64, device="cuda")
        h.Gather(gq, torch.from_numpy(q).cuda(), 1, op, O.Trans)
        np.testing.assert_array_equal(host(gq), orc.gather(rs, ci, q, 1, op))
        dq = torch.from_numpy(q.copy()).cuda()
        h.GatherScatter(dq, 1, op, O.Sym)
        np.testing.assert_array_equal(host(dq), orc.gather_scatter(rs, ci, rs, ci, q, 1, op))


def test_slabs_special_values(cuda, orc, knobs):
    """-0 becomes +0 under Add (the single-member rows store it back); NaN and -Inf
    under Max/Min as the reference's comparisons leave them.  (The sign of a NaN
    made by Inf + -Inf is the host's own -- x86 and Arm differ -- so signs are
    compared where the results are numbers.)"""
    ids = np.array([1, 1, 2, 3, 3, 3, 4, 5, 5, 6], dtype=np.int64)
    h, ref = make(orc, ids)
    v = np.array([-0.0, -0.0, -0.0, np.nan, 1.0, -np.inf, -0.0, np.inf, -np.inf, np.nan])
    for op in (O.Add, O.Max, O.Min, O.Mul):
        dv = torch.from_numpy(v).cuda()
        h.GatherScatter(dv, 1, op, O.Sym)
        want = orc.gather_scatter(ref["rsT"], ref["ciT"], ref["rsT"], ref["ciT"], v, 1, op)
        got = host(dv)
        num = ~np.isnan(want)
        np.testing.assert_array_equal(np.signbit(got[num]), np.signbit(want[num]))
        np.testing.assert_array_equal(got, want)
        gq = torch.zeros(ref["rsT"].size - 1, dtype=torch.float64, device="cuda")
        h.Gather(gq, torch.from_numpy(v).cuda(), 1, op, O.Trans)
        want, got = orc.gather(ref["rsT"], ref["ciT"], v, 1, op), host(gq)
        num = ~np.isnan(want)
        np.testing.assert_array_equal(np.signbit(got[num]), np.signbit(want[num]))
        np.testing.assert_array_equal(got, want)


def test_plan_without_slabs_falls_back(cuda, orc, knobs):
    """Kernel 7 asked of a plan built with ogs.slabs = 0 runs the pipelined chunk
    kernel instead (same bits)."""
    knobs("ogs.slabs", 0)
    ids = O.box_hex_ids(5, 4, 3, 7, 2024)
    h, ref = make(orc, ids)
    assert h.info.NslabsT == 0 and h.info.NslabsGS == 0
    check_fp64(orc, h, ref, ids.size, 3)
