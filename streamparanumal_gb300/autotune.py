"""Per-degree autotuner of the gather-scatter launch configuration.

For a hex box of degree p it times BS6 (Gather Trans), BS7 (Scatter NoTrans) and
BS8 (GatherScatter Sym) under every compiled variant -- block kernels (rows cut into
blocks of `ogs.block_nnz` entries), warp-chunk kernels, pipelined persistent
warp-chunk kernels, asynchronously staged ones and lane-row slabs, each with chunks in row order or
breadth-first page order (whole-mesh wavefronts or chains of balls) and rows in CSR
order or grouped by size -- and keeps the fastest by total time.  The in-place
gather+scatter then gets its own walk of the operator when one of the candidate
walks beats it on the chosen plan.  Results are stored per degree in a JSON table
(`tuning/gb300.json` by default) that :func:`apply` loads into the library's tuning
knobs before plans are built.  Every variant computes the same bits; only speed
differs.
"""
from __future__ import annotations

import json
from pathlib import Path

import torch

from . import capi
from . import ogs as O

TABLE = Path(__file__).resolve().parent / "tuning" / "gb300.json"

# (plan-time knobs) x (launch-time kernel): plans are rebuilt only when order, rows,
# page_shift or block_nnz change
PLAN_CONFIGS = [{"order": 1, "rows": 1, "block_nnz": 2048}, {"order": 1, "rows": 0, "block_nnz": 2048},
                {"order": 0, "rows": 1, "block_nnz": 2048}, {"order": 0, "rows": 0, "block_nnz": 2048},
                {"order": 0, "rows": 0, "block_nnz": 1024}]
DEFAULT_PAGE_SHIFT = 9


BALL_OVER_PAGE = 10  # balls of 2^(page_shift + 10) entries: about a thousand pages


def plan_configs(p: int) -> list[dict]:
    """PLAN_CONFIGS with the default 512-entry pages, plus breadth-first pages of
    about one element ((p+1)^3 entries) when that size differs, plus the
    renumbered breadth-first walk over element-sized pages (chunk order 2); the
    grouped breadth-first configurations also as chains of balls."""
    shift = max(3, ((p + 1) ** 3 - 1).bit_length())
    cfgs = [dict(c, page_shift=DEFAULT_PAGE_SHIFT, ball_shift=0) for c in PLAN_CONFIGS]
    if shift != DEFAULT_PAGE_SHIFT:
        cfgs.insert(1, {"order": 1, "rows": 1, "block_nnz": 2048, "page_shift": shift,
                        "ball_shift": 0})
    cfgs.insert(1, {"order": 2, "rows": 1, "block_nnz": 2048, "page_shift": shift, "ball_shift": 0})
    balls = [dict(c, ball_shift=c["page_shift"] + BALL_OVER_PAGE) for c in cfgs
             if c["order"] >= 1 and c["rows"] == 1]
    return cfgs + balls


def gs_walks(p: int) -> list[dict]:
    """Candidate walks of the in-place gather+scatter: renumbered breadth-first
    walks (chunk order 2) over pages of half and one element, whole-mesh or balls."""
    shift = max(3, ((p + 1) ** 3 - 1).bit_length())
    return [{"gs_order": 2, "gs_page_shift": s, "gs_ball_shift": b}
            for s in sorted({max(3, shift - 1), shift}) for b in (0, s + BALL_OVER_PAGE)]
KERNELS = {0: "block", 1: "warp", 2: "warp-pipelined",
           3: "warp-async-staged gathers / column-order scatter",
           4: "column-order gathers / persistent prefetching column-order scatter",
           5: "pipelined gathers with L2 prefetch of the next chunk / column-major scatter",
           7: "lane-row slabs (gather and gather+scatter)"}
# lane-row slabs (kernel 7) regroup the walk's rows by size inside runs of 2^17
# entries: on the 64^3 p = 7 box 2^16..2^18 measured within 2 % of each other, 2^14
# 9 % and 2^19 and above 30 % slower
SLAB_SEG_SHIFT = 17
OPS = (("BS6", "kernel_gather"), ("BS7", "kernel_scatter"), ("BS8", "kernel_gs"))


def _time(fn, reps: int, stream) -> float:
    for _ in range(2):
        fn()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


KNOBS = {"order": "ogs.order", "rows": "ogs.rows", "page_shift": "ogs.page_shift",
         "block_nnz": "ogs.block_nnz", "ball_shift": "ogs.ball_shift",
         "gs_order": "ogs.gs_order", "gs_page_shift": "ogs.gs_page_shift",
         "gs_ball_shift": "ogs.gs_ball_shift",
         "kernel_gs": "ogs.kernel", "kernel_gather": "ogs.kernel.gather",
         "kernel_scatter": "ogs.kernel.scatter", "scatter_pages": "ogs.scatter_pages",
         "slabs": "ogs.slabs", "slab_seg_shift": "ogs.slab_seg_shift",
         "slab_code_shift": "ogs.slab_code_shift", "kernel_gs32": "ogs.kernel.f32",
         "kernel_gather32": "ogs.kernel.gather.f32"}
# knobs a table entry may leave out: the library defaults
PLAN_DEFAULTS = {"ball_shift": 0, "gs_order": -1, "scatter_pages": 1, "slabs": 0,
                 "slab_seg_shift": SLAB_SEG_SHIFT, "slab_code_shift": 0, "kernel_gs32": -1,
                 "kernel_gather32": -1}


def code_shift(p: int) -> int:
    """Low bits of kernel 7's 16-bit member codes for degree p: enough for the
    (p+1)^3 nodes of an element, so that a code's high part is an element (at
    most 12 bits, p <= 15)."""
    return min(12, max(3, ((p + 1) ** 3 - 1).bit_length()))
GS_WALK_KERNELS = (1, 2, 3, 5, 7)
# the table keys of the operations whose 4-byte kernel is chosen on its own
KEY32 = {"BS6": "kernel_gather32", "BS8": "kernel_gs32"}
# a 4-byte kernel of its own must beat the 8-byte choice's FP32 time by this much
FP32_TIE = 0.02


def _set(cfg: dict) -> None:
    for k, knob in KNOBS.items():
        if k in cfg:
            capi.tune_set(knob, cfg[k])


def _kernels(pc: dict, op: str) -> list[int]:
    """Kernel variants timed under one plan configuration: block kernels ignore the
    chunk order and row grouping, so they run once per block size; the column-order
    scatters ignore the row grouping, so they run under grouped plans only; the
    column-major scatter runs in memory order under the plain plan and over the
    walk's pages under the grouped breadth-first ones."""
    plain = pc["order"] == 0 and pc["rows"] == 0
    ks = [0] if plain else []
    if pc["block_nnz"] == 2048:
        if op == "BS7":
            walked = pc["order"] >= 1 and pc["rows"] == 1
            ks += [1, 2] + ([3, 4] if pc["rows"] == 1 else []) + ([5] if plain or walked else [])
        else:
            ks += [1, 2, 3, 4, 5, 7]
    return ks


def _slabs(choice: dict, p: int | None = None) -> dict:
    """A chosen configuration builds the slab layouts only when a kernel 7 uses them
    (with 16-bit member codes for degree p when p is given)."""
    if 7 in (choice.get("kernel_gather"), choice.get("kernel_gs"), choice.get("kernel_gather32"),
             choice.get("kernel_gs32")):
        choice.update(slabs=1, slab_seg_shift=SLAB_SEG_SHIFT)
        if p is not None:
            choice["slab_code_shift"] = code_shift(p)
    else:
        for k in ("slabs", "slab_seg_shift", "slab_code_shift"):
            choice.pop(k, None)
    return choice


def choose(timings: list[tuple]) -> tuple[dict, float, float]:
    """The winner of the timed candidates (order, rows, page_shift, ball_shift,
    block_nnz, kernel, op, ms): per chunk layout, the fastest kernel of each
    operation; the layout with the least BS6 + BS7 + BS8 time wins (the
    gather+scatter may still get a walk of its own afterwards, which is built with
    the chosen layout's row grouping, so its time on the layout counts too).
    Returns (knobs, BS6 + BS7 ms, BS8 ms).  A candidate may carry a ninth field,
    its time with FP32 values: for BS6 and BS8 the chunk kernel of the chosen
    layout fastest in FP32 becomes the 4-byte kernel (kernel_gather32 /
    kernel_gs32) when it beats the FP64 choice's FP32 time by more than FP32_TIE;
    the FP64 times alone decide the layout and the 8-byte kernels."""
    best_key, best, best_main, best_gs_ms = None, None, None, None
    for layout in sorted({t[:4] for t in timings}):
        order, rows, shift, ball = layout
        choice = {"order": order, "rows": rows, "page_shift": shift, "ball_shift": ball}
        main, gs_ms = 0.0, None
        for op, key in OPS:
            # block kernels and the memory-order column-major scatter (timed under
            # the plain plan) do not depend on the chunk layout, so they compete
            # under every plan configuration
            cands = [t for t in timings if t[6] == op and (
                t[:4] == layout or t[5] == 0 or
                (op == "BS7" and t[5] == 5 and t[0] == 0 and t[1] == 0))]
            win = min(cands, key=lambda t: t[7])
            bnnz, k, ms = win[4], win[5], win[7]
            choice[key] = k
            # 4-byte values may take another chunk kernel of this layout
            c32 = [t for t in cands if len(t) > 8 and t[8] is not None and t[:4] == layout
                   and t[5] >= 1]
            if op in KEY32 and c32:
                b32 = min(c32, key=lambda t: t[8])
                own32 = win[8] if len(win) > 8 and win[8] is not None else None
                # a kernel of its own only when it beats the FP64 choice by the tie band
                if b32[5] != k and (own32 is None or b32[8] * (1.0 + FP32_TIE) < own32):
                    choice[KEY32[op]] = b32[5]
            if op == "BS7" and k == 5:
                choice["scatter_pages"] = int(win[:4] == layout and order >= 1)
            if k == 0 and (op != "BS8" or "block_nnz" not in choice):
                choice["block_nnz"] = bnnz
            if op == "BS8":
                gs_ms = ms
            else:
                main += ms
        if best_key is None or (main + gs_ms, main) < best_key:
            best_key, best, best_main, best_gs_ms = (main + gs_ms, main), choice, main, gs_ms
    best.setdefault("block_nnz", 2048)
    return _slabs(best), best_main, best_gs_ms


def tune_ogs(E: int, p: int, perm_seed: int = 0, dtype=torch.float64, reps: int = 5,
             ids=None) -> dict:
    """Times every variant of BS6 / BS7 / BS8 on an E^3 box of degree p (ids: numpy
    or CUDA tensor; built on the device when omitted); the winner takes, for the
    best (chunk order, row grouping), the fastest kernel of each operation."""
    saved = {k: capi.tune_get(knob) for k, knob in KNOBS.items()}
    stream = torch.cuda.current_stream()
    if ids is None:
        ids = O.box_hex_ids(E, E, E, p, perm_seed, device="cuda")
    Nt = ids.numel() if isinstance(ids, torch.Tensor) else ids.size
    q = torch.rand(Nt, dtype=torch.float64, device="cuda").to(dtype)
    q32 = q.float() if dtype == torch.float64 else None
    # (order, rows, page_shift, ball_shift, block_nnz, kernel, op, ms, FP32 ms or None)
    timings = []
    walk_timings = []  # (gs_order, gs_page_shift, gs_ball_shift, kernel, ms, FP32 ms or None)

    def build():
        h = O.ogs_t()
        h.Setup(Nt, ids.clone() if isinstance(ids, torch.Tensor) else ids.copy(), unique=True)
        return h

    try:
        _set({**PLAN_DEFAULTS, "slabs": 1, "slab_code_shift": code_shift(p)})
        for pc in plan_configs(p):
            _set(pc)
            h = build()
            gq = torch.zeros(h.Ngather, dtype=dtype, device="cuda")
            gq32 = torch.zeros(h.Ngather, dtype=torch.float32, device="cuda") if q32 is not None \
                else None
            ops = {"BS6": lambda: h.Gather(gq, q, 1, O.Add, O.Trans),
                   "BS7": lambda: h.Scatter(q, gq, 1, O.NoTrans),
                   "BS8": lambda: h.GatherScatter(q, 1, O.Add, O.Sym)}
            ops32 = {"BS6": lambda: h.Gather(gq32, q32, 1, O.Add, O.Trans),
                     "BS8": lambda: h.GatherScatter(q32, 1, O.Add, O.Sym)}
            for op, key in OPS:
                for k in _kernels(pc, op):
                    _set({key: k, "scatter_pages": 1})
                    ms32 = _time(ops32[op], reps, stream) if q32 is not None and op in ops32 \
                        else None
                    timings.append((pc["order"], pc["rows"], pc["page_shift"], pc["ball_shift"],
                                    pc["block_nnz"], k, op, _time(ops[op], reps, stream), ms32))
            h.Free()
            del gq, gq32
        # the main walk serves the gathers and scatters; the gather+scatter may get
        # a walk of its own below, so it decides the main walk only on a tie
        best, main_ms, best_gs_ms = choose(timings)
        best_total = main_ms + best_gs_ms
        # a walk of its own for the gather+scatter, on the chosen plan
        if best["order"] != 0 or best["rows"] != 0 or best.get("kernel_gs", 0) != 0:
            for w in gs_walks(p):
                _set({**best, **w})
                h = build()
                for k in GS_WALK_KERNELS:
                    _set({"kernel_gs": k})
                    ms32 = _time(lambda: h.GatherScatter(q32, 1, O.Add, O.Sym), reps, stream) \
                        if q32 is not None else None
                    walk_timings.append((w["gs_order"], w["gs_page_shift"], w["gs_ball_shift"], k,
                                         _time(lambda: h.GatherScatter(q, 1, O.Add, O.Sym), reps,
                                               stream), ms32))
                h.Free()
        best["gs_order"] = -1
        if walk_timings:
            # the chosen layout's own gather+scatter against the walks, by FP64 time
            cands = [(t[4], t[5], t[:4]) for t in walk_timings]
            cands.append((best_gs_ms, None, None))
            win = min(cands, key=lambda c: c[0])
            if win[2] is not None:
                go, gp, gb, k = win[2]
                best.update(gs_order=go, gs_page_shift=gp, gs_ball_shift=gb, kernel_gs=k)
                best_total += win[0] - best_gs_ms
                # the 4-byte gather+scatter takes the fastest kernel on that walk
                w32 = [t for t in walk_timings if t[:3] == (go, gp, gb) and t[5] is not None]
                best.pop("kernel_gs32", None)
                if w32:
                    b32 = min(w32, key=lambda t: t[5])
                    own32 = next((t[5] for t in w32 if t[3] == k), None)
                    if b32[3] != k and (own32 is None or b32[5] * (1.0 + FP32_TIE) < own32):
                        best["kernel_gs32"] = b32[3]
        _slabs(best, p)
    finally:
        _set(saved)
    return {"p": p, "E": E, "perm": bool(perm_seed), "local_nodes": int(Nt), "best": best,
            "best_total_ms": best_total,
            "candidates": [{"order": o, "rows": r, "page_shift": ps, "ball_shift": bs,
                            "block_nnz": b, "kernel": k, "op": op, "ms": ms, "ms_fp32": ms32}
                           for o, r, ps, bs, b, k, op, ms, ms32 in timings],
            "gs_walks": [{"gs_order": o, "gs_page_shift": ps, "gs_ball_shift": bs, "kernel": k,
                          "ms": ms, "ms_fp32": ms32} for o, ps, bs, k, ms, ms32 in walk_timings]}


def load_table(path: Path = TABLE) -> dict:
    if path.exists():
        return json.loads(path.read_text())
    return {}


def save_table(table: dict, path: Path = TABLE) -> None:
    """Writes the table as JSON and, beside it, the text form the BS6-BS8 drivers
    read (one line per key: `p7_perm ogs.order=1 ogs.rows=1 ...`)."""
    path.parent.mkdir(parents=True, exist_ok=True)
    path.write_text(json.dumps(table, indent=1, sort_keys=True) + "\n")
    path.with_suffix(".txt").write_text(table_text(table))


def table_text(table: dict) -> str:
    lines = []
    for key in sorted(table):
        cfg = table[key]
        lines.append(" ".join([key] + [f"{KNOBS[k]}={int(cfg[k])}" for k in sorted(cfg)
                                       if k in KNOBS]))
    return "\n".join(lines) + "\n"


def record(table: dict, result: dict) -> None:
    """Stores a tune_ogs() winner under its degree (and layout)."""
    key = f"p{result['p']}" + ("_perm" if result["perm"] else "")
    table[key] = result["best"]


def apply(p: int, perm: bool = False, table: dict | None = None) -> dict:
    """Sets the ogs knobs for degree p from the table (library defaults when the
    degree is not tuned); plans created afterwards use them."""
    table = load_table() if table is None else table
    cfg = table.get(f"p{p}" + ("_perm" if perm else "")) or table.get(f"p{p}")
    if cfg:
        _set({**PLAN_DEFAULTS, **cfg})
    return cfg or {}
