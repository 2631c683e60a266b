"""Per-degree autotuner of the gather-scatter launch configuration.

For a hex box of degree p it times BS6 (Gather Trans), BS7 (Scatter NoTrans) and
BS8 (GatherScatter Sym) under every compiled variant -- block kernels (rows cut into
blocks of `ogs.block_nnz` entries), warp-chunk kernels, pipelined persistent
warp-chunk kernels and asynchronously staged ones, each with chunks in row order or
breadth-first page order and rows in CSR order or grouped by size -- and keeps the
fastest by total time.  Results are stored per degree in a JSON table
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


def plan_configs(p: int) -> list[dict]:
    """PLAN_CONFIGS with the default 512-entry pages, plus breadth-first pages of
    about one element ((p+1)^3 entries) when that size differs, plus the
    renumbered breadth-first walk over element-sized pages (chunk order 2)."""
    shift = max(3, ((p + 1) ** 3 - 1).bit_length())
    cfgs = [dict(c, page_shift=DEFAULT_PAGE_SHIFT) for c in PLAN_CONFIGS]
    if shift != DEFAULT_PAGE_SHIFT:
        cfgs.insert(1, {"order": 1, "rows": 1, "block_nnz": 2048, "page_shift": shift})
    cfgs.insert(1, {"order": 2, "rows": 1, "block_nnz": 2048, "page_shift": shift})
    return cfgs
KERNELS = {0: "block", 1: "warp", 2: "warp-pipelined",
           3: "warp-async-staged gathers / column-order scatter",
           4: "column-order gathers / persistent prefetching column-order scatter",
           5: "pipelined gathers with L2 prefetch of the next chunk / column-major scatter"}
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
         "block_nnz": "ogs.block_nnz",
         "kernel_gs": "ogs.kernel", "kernel_gather": "ogs.kernel.gather",
         "kernel_scatter": "ogs.kernel.scatter"}


def _set(cfg: dict) -> None:
    for k, knob in KNOBS.items():
        if k in cfg:
            capi.tune_set(knob, cfg[k])


def _kernels(pc: dict, op: str) -> list[int]:
    """Kernel variants timed under one plan configuration: block kernels ignore the
    chunk order and row grouping, so they run once per block size; the column-order
    scatters ignore the row grouping, so they run under grouped plans only."""
    plain = pc["order"] == 0 and pc["rows"] == 0
    ks = [0] if plain else []
    if pc["block_nnz"] == 2048:
        if op == "BS7":
            # the column-major scatter (5) ignores chunks: timed once, with the plain plan
            ks += [1, 2] + ([3, 4] if pc["rows"] == 1 else []) + ([5] if plain else [])
        else:
            ks += [1, 2, 3, 4, 5]
    return ks


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
    timings = []  # (order, rows, page_shift, block_nnz, kernel, op, ms)
    try:
        for pc in plan_configs(p):
            _set(pc)
            h = O.ogs_t()
            h.Setup(Nt, ids.clone() if isinstance(ids, torch.Tensor) else ids.copy(), unique=True)
            gq = torch.zeros(h.Ngather, dtype=dtype, device="cuda")
            ops = {"BS6": lambda: h.Gather(gq, q, 1, O.Add, O.Trans),
                   "BS7": lambda: h.Scatter(q, gq, 1, O.NoTrans),
                   "BS8": lambda: h.GatherScatter(q, 1, O.Add, O.Sym)}
            for op, key in OPS:
                for k in _kernels(pc, op):
                    _set({key: k})
                    timings.append((pc["order"], pc["rows"], pc["page_shift"], pc["block_nnz"], k,
                                    op, _time(ops[op], reps, stream)))
            h.Free()
            del gq
    finally:
        _set(saved)
    best_total, best = None, None
    for order, rows, shift in sorted({t[:3] for t in timings}):
        choice, total = {"order": order, "rows": rows, "page_shift": shift}, 0.0
        for op, key in OPS:
            # block kernels and the column-major scatter do not depend on the chunk
            # layout, so they compete under every plan configuration
            cands = [t for t in timings if t[5] == op and (
                t[:3] == (order, rows, shift) or t[4] == 0 or (op == "BS7" and t[4] == 5))]
            _, _, _, bnnz, k, _, ms = min(cands, key=lambda t: t[6])
            choice[key] = k
            if k == 0:
                choice["block_nnz"] = bnnz
            total += ms
        if best_total is None or total < best_total:
            best_total, best = total, choice
    best.setdefault("block_nnz", 2048)
    return {"p": p, "E": E, "perm": bool(perm_seed), "local_nodes": int(Nt), "best": best,
            "best_total_ms": best_total,
            "candidates": [{"order": o, "rows": r, "page_shift": ps, "block_nnz": b, "kernel": k,
                            "op": op, "ms": ms} for o, r, ps, b, k, op, ms in timings]}


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
        _set(cfg)
    return cfg or {}
