"""Generate the golden fixtures from the reference's own code.

Runs oracle/_ref/refdump -- the reference's host code (mesh_t, ogs_t, prim::)
compiled from its sources with the single-rank MPI and host-only OCCA stand-ins,
plus its BS1-BS5 OKL kernels lowered for OCCA Serial execution -- and records
SHA-256 digests and a few leading values of every output, together with the
inputs' seeds, in tests/golden/*.json.  Small cases also keep the reference's
signed ids (after its unique-owner flagging) so the N-operator paths can be
checked against the reference's own owners.  The multi-rank cases run the
reference on several forked ranks that meet through the MPI stand-in of
oracle/ref/shim/mpi.h.

Needs the reference tree (build with `make -C oracle/ref REF=<reference tree>`); the committed fixtures
are what the tests read.  Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
REFDUMP = ROOT / "oracle" / "_ref" / "refdump"

# (nx, ny, nz, p, perm_seed, qseed)
OGS_CASES = [
    (3, 2, 2, 3, 0, 77),
    (2, 3, 2, 2, 5, 78),
    (1, 1, 1, 1, 0, 79),
    (5, 1, 2, 4, 0, 80),
    (4, 4, 4, 7, 0, 81),
    (4, 4, 4, 7, 99, 82),
    (6, 5, 4, 5, 2024, 83),
    (16, 16, 16, 7, 0, 2024),   # BS8 anchor configuration: 2,097,152 local nodes
]
KEEP_IDS_MAX = 40000
# multi-rank: (ranks, nx, ny, nz, p, qseed), nx*ny*nz elements per rank.  Rank counts
# are powers of two: the reference's mesh setup also builds its CrystalRouter
# exchange (Auto method), whose setup leaves messages unmatched at other counts.
OGSMR_CASES = [
    (2, 2, 2, 2, 2, 31),
    (4, 2, 3, 2, 3, 32),
    (8, 2, 2, 2, 2, 33),
    (2, 3, 3, 3, 5, 34),
]
OGSMR_OUTPUTS = ["gs_sym", "gs_notrans", "gs_trans", "gs_sym_max", "gather_sym",
                 "gather_notrans", "gather_trans", "scatter_sym", "scatter_notrans",
                 "scatter_trans"]
BS_CASES = [(1, 11), (5, 12), (1000, 13), (65537, 14), (300001, 15), (1048576, 16)]


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def hexes(a: np.ndarray, n: int = 8) -> list[str]:
    return [float(x).hex() for x in a[:n]]


def run(args, out):
    subprocess.run([str(REFDUMP), *map(str, args), str(out)], check=True, capture_output=True)


def ogs_case(nx, ny, nz, p, perm, qseed):
    with tempfile.TemporaryDirectory() as d:
        run(["ogs", nx, ny, nz, p, perm, qseed], d)
        ld = lambda n, t: np.fromfile(f"{d}/{n}.bin", dtype=t)  # noqa: E731
        ids = ld("ids", np.int64)
        row_of = ld("row_of", np.int64)
        rec = {"mesh": [nx, ny, nz, p], "perm_seed": perm, "qseed": qseed, "N": int(ids.size),
               "Ngather": int(row_of.max()) + 1 if row_of.size else 0,
               "sha256": {"abs_ids_rows": sha(row_of), "ids_signed": sha(ids)}, "head": {}}
        for name in ("q", "gs_sym", "gather_trans", "gather_notrans", "scatter_notrans"):
            a = ld(name, np.float64)
            rec["sha256"][name] = sha(a)
            rec["head"][name] = hexes(a)
        stem = f"ogs_{nx}x{ny}x{nz}_p{p}_s{perm}"
        if ids.size <= KEEP_IDS_MAX:
            np.save(HERE / f"{stem}_ids.npy", ids)
            rec["ids_file"] = f"{stem}_ids.npy"
        (HERE / f"{stem}.json").write_text(json.dumps(rec, indent=1) + "\n")
        print(stem, rec["N"], rec["Ngather"])


def ogsmr_case(size, nx, ny, nz, p, qseed):
    """The reference's ogs_t on `size` ranks (forked, MPI stand-in): per rank the box
    ids, its signed ids after the mesh's unique flagging, the counts of a Pairwise
    handle on those ids and digests of its operations on seeded values."""
    with tempfile.TemporaryDirectory() as d:
        run(["ogsmr", size, nx, ny, nz, p, qseed], d)
        ranks, ids = [], {}
        for r in range(size):
            ld = lambda n, t: np.fromfile(f"{d}/r{r}_{n}.bin", dtype=t)  # noqa: E731
            cnt = ld("counts", np.int64)
            rec = {"counts": dict(zip(["N", "NlocalP", "NlocalT", "NhaloP", "NhaloT", "Ngather",
                                       "NgatherGlobal", "gather_defined"], map(int, cnt))),
                   "sha256": {"box_ids": sha(ld("box_ids", np.int64))}, "head": {}}
            ids[f"r{r}"] = ld("ids", np.int64)
            for name in OGSMR_OUTPUTS:
                a = ld(name, np.float64)
                rec["sha256"][name] = sha(a)
                rec["head"][name] = hexes(a)
            ranks.append(rec)
        stem = f"ogsmr_{size}r_{nx}x{ny}x{nz}_p{p}"
        np.savez_compressed(HERE / f"{stem}_ids.npz", **ids)
        case = {"ranks": size, "mesh": [nx, ny, nz, p], "qseed": qseed,
                "q_seed_of_rank": "qseed + 1000*rank", "g_seed_of_rank": "qseed + 1000*rank + 1",
                "ids_file": f"{stem}_ids.npz", "per_rank": ranks}
        (HERE / f"{stem}.json").write_text(json.dumps(case, indent=1) + "\n")
        print(stem, [r["counts"]["NhaloT"] for r in ranks])


def bs_case(n, seed):
    with tempfile.TemporaryDirectory() as d:
        run(["bs", n, seed], d)
        rec = {"N": n, "seed": seed, "alpha": -0.7353, "beta": 0.4142,
               "fp_contract": "off (OCCA Serial)", "sha256": {}, "value": {}}
        for name in ("bs1", "bs2", "bs5_r", "bs3_partial", "bs4_partial", "bs5_partial"):
            rec["sha256"][name] = sha(np.fromfile(f"{d}/{name}.bin", dtype=np.float64))
        for name in ("bs3", "bs4", "bs5", "bs5_256"):
            rec["value"][name] = float(np.fromfile(f"{d}/{name}.bin", dtype=np.float64)[0]).hex()
        (HERE / f"bs_n{n}.json").write_text(json.dumps(rec, indent=1) + "\n")
        print("bs", n)


def main():
    if not REFDUMP.exists():
        sys.exit("oracle/_ref/refdump missing: run `make -C oracle/ref REF=<reference tree>`")
    for c in OGS_CASES:
        ogs_case(*c)
    for c in BS_CASES:
        bs_case(*c)
    for c in OGSMR_CASES:
        ogsmr_case(*c)


if __name__ == "__main__":
    main()
