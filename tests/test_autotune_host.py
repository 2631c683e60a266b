"""The autotuner's host logic (no GPU): plan configurations per degree, the kernel
candidates of each, and the tuning table round trip."""
import json

from streamparanumal_gb300 import autotune


def test_plan_configs_add_element_pages_renumbered_walk_and_balls():
    # p = 7: an element is 512 entries, the default page size
    cfgs = autotune.plan_configs(7)
    assert {(c["order"], c["rows"], c["page_shift"], c["ball_shift"]) for c in cfgs} >= {
        (1, 1, 9, 0), (2, 1, 9, 0), (1, 0, 9, 0), (0, 1, 9, 0), (0, 0, 9, 0), (1, 1, 9, 19),
        (2, 1, 9, 19)}
    assert len(cfgs) == len(autotune.PLAN_CONFIGS) + 1 + 2
    # p = 3: 64-entry elements add pages of 2^6 for both breadth-first orders, and
    # every grouped breadth-first layout also runs as a chain of balls
    cfgs = autotune.plan_configs(3)
    assert {"order": 1, "rows": 1, "block_nnz": 2048, "page_shift": 6, "ball_shift": 0} in cfgs
    assert {"order": 2, "rows": 1, "block_nnz": 2048, "page_shift": 6, "ball_shift": 16} in cfgs
    assert len(cfgs) == len(autotune.PLAN_CONFIGS) + 2 + 3
    # p = 1: 8-entry elements
    assert min(c["page_shift"] for c in autotune.plan_configs(1)) == 3


def test_gather_scatter_walk_candidates():
    assert autotune.gs_walks(7) == [
        {"gs_order": 2, "gs_page_shift": 8, "gs_ball_shift": 0},
        {"gs_order": 2, "gs_page_shift": 8, "gs_ball_shift": 18},
        {"gs_order": 2, "gs_page_shift": 9, "gs_ball_shift": 0},
        {"gs_order": 2, "gs_page_shift": 9, "gs_ball_shift": 19}]
    assert {w["gs_page_shift"] for w in autotune.gs_walks(1)} == {3}


def test_kernel_candidates():
    grouped = {"order": 1, "rows": 1, "block_nnz": 2048, "page_shift": 9}
    plain_rows = {"order": 0, "rows": 0, "block_nnz": 2048, "page_shift": 9}
    small_blocks = {"order": 0, "rows": 0, "block_nnz": 1024, "page_shift": 9}
    assert autotune._kernels(grouped, "BS6") == [1, 2, 3, 4, 5, 7]
    assert autotune._kernels(grouped, "BS7") == [1, 2, 3, 4, 5]
    assert autotune._kernels(dict(grouped, rows=0), "BS7") == [1, 2]
    assert autotune._kernels(plain_rows, "BS8") == [0, 1, 2, 3, 4, 5, 7]
    assert autotune._kernels(plain_rows, "BS7") == [0, 1, 2, 5]
    assert autotune._kernels(small_blocks, "BS6") == [0]


def test_table_round_trip(tmp_path):
    table = {}
    autotune.record(table, {"p": 5, "perm": True, "best": {"order": 2, "rows": 1,
                                                              "page_shift": 8}})
    autotune.record(table, {"p": 5, "perm": False, "best": {"order": 0, "rows": 1}})
    path = tmp_path / "t.json"
    autotune.save_table(table, path)
    assert json.loads(path.read_text()) == table
    assert autotune.load_table(path) == table
    assert autotune.load_table(tmp_path / "missing.json") == {}


def test_committed_table_is_well_formed():
    table = autotune.load_table()
    assert table, "the committed GB300 tuning table is missing"
    for key, cfg in table.items():
        assert key.startswith("p")
        assert set(cfg) <= set(autotune.KNOBS)
        assert cfg["order"] in (0, 1, 2) and cfg["kernel_gs"] in (0, 1, 2, 3, 4, 5, 7)
        # the slab layouts are built exactly where a kernel 7 runs on them
        uses = 7 in (cfg["kernel_gather"], cfg["kernel_gs"], cfg.get("kernel_gather32"),
                     cfg.get("kernel_gs32"))
        assert cfg.get("slabs", 0) == int(uses)
        p = int(key[1:].split("_")[0])
        assert cfg.get("slab_code_shift", 0) == (autotune.code_shift(p) if uses else 0)


def test_text_form_matches_the_table():
    """The drivers read the text form; it carries the same knobs as the JSON."""
    table = autotune.load_table()
    txt = autotune.TABLE.with_suffix(".txt").read_text()
    assert txt == autotune.table_text(table)
    line = next(ln for ln in txt.splitlines() if ln.split()[0] == "p7_perm")
    fields = dict(f.split("=") for f in line.split()[1:])
    assert {autotune.KNOBS[k]: str(v) for k, v in table["p7_perm"].items()} == fields


def _timings(ms: dict) -> list[tuple]:
    """Synthetic timings: every candidate of plan_configs(7) at 1 ms unless listed in
    ms ((order, rows, page_shift, ball_shift, block_nnz, kernel, op) -> ms)."""
    out = []
    for pc in autotune.plan_configs(7):
        for op, _ in autotune.OPS:
            for k in autotune._kernels(pc, op):
                key = (pc["order"], pc["rows"], pc["page_shift"], pc["ball_shift"],
                       pc["block_nnz"], k, op)
                out.append(key + (ms.get(key, 1.0),))
    return out


def test_choose_walk_ordered_scatter_stays_with_its_layout():
    walk = (1, 1, 9, 19, 2048)
    best, main, gs = autotune.choose(_timings({
        walk + (2, "BS6"): 0.5, walk + (5, "BS7"): 0.4, walk + (2, "BS8"): 0.6,
        (0, 0, 9, 0, 2048, 5, "BS7"): 0.45}))
    assert (best["order"], best["rows"], best["page_shift"], best["ball_shift"]) == walk[:4]
    assert best["kernel_gather"] == 2 and best["kernel_scatter"] == 5
    assert best["scatter_pages"] == 1 and main == 0.9 and gs == 0.6


def test_choose_memory_order_scatter_competes_under_every_layout():
    walk = (1, 1, 9, 19, 2048)
    best, main, _ = autotune.choose(_timings({
        walk + (2, "BS6"): 0.5, walk + (5, "BS7"): 0.7,
        (0, 0, 9, 0, 2048, 5, "BS7"): 0.45}))
    assert best["ball_shift"] == 19 and best["kernel_scatter"] == 5
    assert best["scatter_pages"] == 0 and main == 0.95
    # a walk-ordered scatter of another layout does not compete here
    best, _, _ = autotune.choose(_timings({
        walk + (2, "BS6"): 0.5, (2, 1, 9, 0, 2048, 5, "BS7"): 0.1}))
    assert best["order"] == 2 and best["scatter_pages"] == 1


def test_choose_block_kernels_keep_their_block_size():
    best, _, _ = autotune.choose(_timings({(0, 0, 9, 0, 1024, 0, "BS6"): 0.2,
                                           (0, 0, 9, 0, 2048, 5, "BS7"): 0.5}))
    assert best["kernel_gather"] == 0 and best["block_nnz"] == 1024
    assert best["kernel_scatter"] == 5 and best["scatter_pages"] == 0


def test_choose_lane_row_slabs_builds_their_layout():
    walk = (1, 1, 9, 19, 2048)
    best, _, _ = autotune.choose(_timings({walk + (7, "BS6"): 0.5, walk + (5, "BS7"): 0.5,
                                           walk + (2, "BS8"): 0.5}))
    assert best["kernel_gather"] == 7 and best["kernel_gs"] == 2
    assert best["slabs"] == 1 and best["slab_seg_shift"] == autotune.SLAB_SEG_SHIFT
    best, _, _ = autotune.choose(_timings({walk + (2, "BS6"): 0.5, walk + (5, "BS7"): 0.5}))
    assert 7 not in (best["kernel_gather"], best["kernel_gs"]) and "slabs" not in best


def test_choose_counts_the_gather_scatter_time_of_each_layout():
    # the plain layout is a little faster for BS6 + BS7 but its gather+scatter is
    # slow; the grouped walk wins on the three together
    walk, plain = (1, 1, 9, 19, 2048), (0, 0, 9, 0, 2048)
    best, main, gs = autotune.choose(_timings({
        plain + (7, "BS6"): 0.40, plain + (5, "BS7"): 0.40, plain + (1, "BS8"): 0.9,
        walk + (7, "BS6"): 0.45, walk + (5, "BS7"): 0.45, walk + (2, "BS8"): 0.5}))
    assert (best["order"], best["rows"], best["ball_shift"]) == (1, 1, 19)
    # (BS7 takes the memory-order column-major scatter of the plain plan, which
    # competes under every layout)
    assert best["kernel_gs"] == 2 and abs(main - 0.85) < 1e-12 and gs == 0.5


def test_code_shift_covers_an_element():
    assert [autotune.code_shift(p) for p in (1, 2, 3, 5, 7, 9, 15)] == [3, 5, 6, 8, 9, 10, 12]
    for p in range(1, 16):
        assert (p + 1) ** 3 <= 1 << autotune.code_shift(p)


def test_choose_fp64_decides_the_8byte_kernel_fp32_its_own():
    walk = (1, 1, 9, 19, 2048)
    t = [x + (None,) for x in _timings({walk + (2, "BS6"): 0.500, walk + (7, "BS6"): 0.505})]
    t = [x[:8] + ((0.30 if x[5] == 7 else 0.40),) if x[:7] in (walk + (2, "BS6"), walk + (7, "BS6"))
         else x for x in t]
    best, _, _ = autotune.choose(t)
    assert best["kernel_gather"] == 2 and best["kernel_gather32"] == 7 and best["slabs"] == 1
    # within the band FP32 keeps the 8-byte kernel
    t = [x[:8] + ((0.395 if x[5] == 7 else 0.40),) if x[:7] in (walk + (2, "BS6"), walk + (7, "BS6"))
         else x for x in t]
    best, _, _ = autotune.choose(t)
    assert best["kernel_gather"] == 2 and "kernel_gather32" not in best and "slabs" not in best


def test_choose_takes_a_4byte_kernel_of_its_own():
    walk = (1, 1, 9, 19, 2048)
    t = [x + (1.0,) for x in _timings({walk + (2, "BS6"): 0.5, walk + (2, "BS8"): 0.5})]
    # FP64 prefers kernel 2 by far; FP32 runs kernel 7 fastest on this layout
    t = [x[:8] + (0.2,) if x[:7] in (walk + (7, "BS6"), walk + (7, "BS8")) else x for x in t]
    best, _, _ = autotune.choose(t)
    assert best["kernel_gather"] == 2 and best["kernel_gather32"] == 7
    assert best["kernel_gs"] == 2 and best["kernel_gs32"] == 7 and best["slabs"] == 1
    # no separate key when FP32's winner is the FP64 one
    t = [x[:8] + (1.0,) for x in t]
    best, _, _ = autotune.choose(t)
    assert "kernel_gather32" not in best and "kernel_gs32" not in best
