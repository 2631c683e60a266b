"""Multi-rank gather-scatter on the host (no GPU): the setup of sp_ogs_mr_setup over
several ranks (threads of this process, or gloo processes), its operators and
exchange schedules checked by running the reference's data flow on the CPU
(tests/mr_emul.py) against

* the reference's own multi-rank ogs_t, run on forked ranks through the MPI
  stand-in (fixtures tests/golden/ogsmr_*.json, made by make_golden.py), bit for bit;
* at rank counts the fixtures do not cover, the one-rank gather-scatter over all
  ranks' nodes together (exact for integers).
"""
import ctypes
import hashlib
import json
import socket
from pathlib import Path

import numpy as np
import pytest

import mr_emul as M
from streamparanumal_gb300 import capi
from streamparanumal_gb300 import comm as C
from streamparanumal_gb300 import ogs as O

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = sorted(GOLDEN.glob("ogsmr_*r_*.json"))
OUTS = ["gs_sym", "gs_notrans", "gs_trans", "gs_sym_max", "gather_sym", "gather_notrans",
        "gather_trans", "scatter_sym", "scatter_notrans", "scatter_trans"]


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def load_case(path):
    case = json.loads(path.read_text())
    z = np.load(GOLDEN / case["ids_file"])
    ids = [z[f"r{r}"].copy() for r in range(case["ranks"])]
    return case, ids


def run_outputs(hh, orc, case, P):
    """Every output of the fixture, per rank, from the emulated data flow."""
    out = {}
    q = [orc.uniform(hh[r].N, case["qseed"] + 1000 * r) for r in range(P)]
    g = [orc.uniform(hh[r].NlocalT + hh[r].NhaloT, case["qseed"] + 1000 * r + 1) for r in range(P)]
    for m, name in ((O.Sym, "sym"), (O.NoTrans, "notrans"), (O.Trans, "trans")):
        ex = M.thread_exchanges(P)
        out["gs_" + name] = C.run_threads(
            P, lambda c: M.gather_scatter(hh[c.rank], orc, q[c.rank], 1, capi.ADD, m, ex[c.rank]))
        ex = M.thread_exchanges(P)
        gv = C.run_threads(P, lambda c: M.gather(hh[c.rank], orc, q[c.rank], 1, capi.ADD, m,
                                                 ex[c.rank]))
        # the reference's buffer holds NlocalT + NhaloT rows, unused rows zero
        out["gather_" + name] = [np.concatenate([a, np.zeros(g[r].size - a.size)])
                                 for r, a in enumerate(gv)]
        ex = M.thread_exchanges(P)
        out["scatter_" + name] = C.run_threads(
            P, lambda c: M.scatter(hh[c.rank], orc, np.zeros(hh[c.rank].N), g[c.rank], 1, m,
                                   ex[c.rank]))
    ex = M.thread_exchanges(P)
    out["gs_sym_max"] = C.run_threads(
        P, lambda c: M.gather_scatter(hh[c.rank], orc, q[c.rank], 1, capi.MAX, O.Sym, ex[c.rank]))
    return out


@pytest.mark.parametrize("path", CASES, ids=[p.stem for p in CASES])
def test_box_ids_of_each_rank_match_the_reference(lib, path):
    case, _ = load_case(path)
    nx, ny, nz, p = case["mesh"]
    P = case["ranks"]
    for r in range(P):
        mine = O.box_hex_ids(nx, ny, nz, p, 0, size=P, rank=r)
        assert sha(mine) == case["per_rank"][r]["sha256"]["box_ids"], f"rank {r}"


@pytest.mark.parametrize("path", CASES, ids=[p.stem for p in CASES])
def test_multi_rank_setup_and_exchange_match_the_reference(lib, orc, path):
    """With the reference's owner flags (its signed ids), counts and every output of
    the reference's Pairwise handle are reproduced bit for bit, FP64 sums included."""
    case, ids = load_case(path)
    P = case["ranks"]
    N = ids[0].size
    hh = C.run_threads(P, lambda c: M.HostHandle(N, ids[c.rank], c, capi.SIGNED, False))
    try:
        for r, h in enumerate(hh):
            want = case["per_rank"][r]["counts"]
            got = {"N": h.N, "NlocalP": h.NlocalP, "NlocalT": h.NlocalT, "NhaloP": h.NhaloP,
                   "NhaloT": h.NhaloT, "Ngather": h.info.Ngather,
                   "NgatherGlobal": h.info.NgatherGlobal, "gather_defined": h.info.gather_defined}
            assert got == want, f"rank {r}"
        out = run_outputs(hh, orc, case, P)
        for name in OUTS:
            for r in range(P):
                assert sha(out[name][r]) == case["per_rank"][r]["sha256"][name], (name, r)
    finally:
        for h in hh:
            h.close()


def _global_check(orc, ids, hh, P, dtype, op=capi.ADD, k=1, seed=5):
    """Multi-rank GatherScatter of every mode against the one-rank operator over all
    ranks' nodes together."""
    allids = np.concatenate(ids)
    g = orc.ogs_setup(allids.copy(), 1, False)
    rsNp = np.concatenate([g["rsN"], np.full(g["rsT"].size - g["rsN"].size, g["rsN"][-1],
                                             dtype=np.int32)])
    cases = {O.Sym: (g["rsT"], g["ciT"], g["rsT"], g["ciT"]),
             O.NoTrans: (rsNp, g["ciN"], g["rsT"], g["ciT"]),
             O.Trans: (g["rsT"], g["ciT"], rsNp, g["ciN"])}
    rng = np.random.default_rng(seed)
    vals = [rng.integers(-9, 10, ids[r].size * k).astype(dtype) for r in range(P)]
    for trans, csr in cases.items():
        ex = M.thread_exchanges(P)
        got = np.concatenate(C.run_threads(P, lambda c: M.gather_scatter(
            hh[c.rank], orc, vals[c.rank], k, op, trans, ex[c.rank])))
        want = orc.gather_scatter(*csr, np.concatenate(vals), k, op)
        np.testing.assert_array_equal(got, want, err_msg=f"trans={trans} op={op}")


@pytest.mark.parametrize("P,box", [(3, (2, 2, 2, 3)), (5, (2, 1, 3, 2)), (6, (1, 2, 2, 3)),
                                   (7, (1, 1, 2, 2))])
def test_any_rank_count_matches_one_rank_operator(lib, orc, P, box):
    """Rank counts that are not powers of two: own owner draws (unique), then every
    mode against the one-rank gather-scatter of all nodes (integers: exact)."""
    nx, ny, nz, p = box
    ids = [O.box_hex_ids(nx, ny, nz, p, 0, size=P, rank=r) for r in range(P)]
    N = ids[0].size
    hh = C.run_threads(P, lambda c: M.HostHandle(N, ids[c.rank], c, capi.SIGNED, True))
    try:
        # unique: exactly one positive copy of every id over all ranks
        allids = np.concatenate(ids)
        pos = np.bincount(allids[allids > 0], minlength=np.abs(allids).max() + 1)
        assert set(np.unique(pos[np.unique(np.abs(allids))])) == {1}
        assert sum(h.NlocalP + h.NhaloP for h in hh) == np.unique(np.abs(allids)).size
        assert all(h.info.NgatherGlobal == np.unique(np.abs(allids)).size for h in hh)
        _global_check(orc, ids, hh, P, np.int64)
        _global_check(orc, ids, hh, P, np.int32, op=capi.MAX, k=2)
        _global_check(orc, ids, hh, P, np.int64, op=capi.MIN, k=3)
    finally:
        for h in hh:
            h.close()


def test_scattered_ids_and_undefined_gather(lib, orc):
    """Ids spread at random over 3 ranks, zeros and arbitrary signs (no unique):
    groups with several or no positive copies make the gather undefined on every
    rank; the Sym gather-scatter still equals the one-rank operator."""
    P, N = 3, 700
    rng = np.random.default_rng(11)
    ids = []
    for r in range(P):
        a = rng.integers(1, 400, N).astype(np.int64)
        a[rng.random(N) < 0.4] *= -1
        a[rng.random(N) < 0.1] = 0
        ids.append(a)
    hh = C.run_threads(P, lambda c: M.HostHandle(N, ids[c.rank], c, capi.SIGNED, False))
    try:
        assert {h.info.gather_defined for h in hh} == {0}
        allids = np.concatenate(ids)
        g = orc.ogs_setup(allids.copy(), 1, False)
        rng2 = np.random.default_rng(3)
        vals = [rng2.integers(-100, 100, N).astype(np.int64) for _ in range(P)]
        ex = M.thread_exchanges(P)
        got = np.concatenate(C.run_threads(P, lambda c: M.gather_scatter(
            hh[c.rank], orc, vals[c.rank], 1, capi.ADD, O.Sym, ex[c.rank])))
        np.testing.assert_array_equal(
            got, orc.gather_scatter(g["rsT"], g["ciT"], g["rsT"], g["ciT"], np.concatenate(vals)))
    finally:
        for h in hh:
            h.close()


def test_unsigned_kind_shares_one_schedule(lib, orc):
    P = 2
    ids = [O.box_hex_ids(2, 2, 1, 2, 0, size=P, rank=r) for r in range(P)]
    N = ids[0].size
    hh = C.run_threads(P, lambda c: M.HostHandle(N, ids[c.rank], c, capi.UNSIGNED, False))
    try:
        for h in hh:
            s = [h.sched[m] for m in M.MODES]
            assert s[0].Nsend == s[1].Nsend == s[2].Nsend == h.info.Nshared
            assert s[0].Nrows == s[1].Nrows == s[2].Nrows == h.NhaloT
        _global_check(orc, ids, hh, P, np.int64)
    finally:
        for h in hh:
            h.close()


def test_single_rank_equals_one_rank_setup(lib):
    ids = O.box_hex_ids(3, 2, 2, 3)
    h = C.run_threads(1, lambda c: M.HostHandle(ids.size, ids.copy(), c, capi.SIGNED, True))[0]
    try:
        assert h.NhaloT == 0 and h.info.Nshared == 0
        ref = ids.copy()
        nT, nN = ctypes.c_int32(), ctypes.c_int32()
        rsT = np.zeros(ids.size + 1, np.int32)
        ciT = np.zeros(ids.size, np.int32)
        rsN = np.zeros(ids.size + 1, np.int32)
        ciN = np.zeros(ids.size, np.int32)
        capi.call("sp_ogs_setup_csr", ids.size, capi.i64p(ref), capi.SIGNED, 1, ctypes.byref(nT),
                  capi.i32p(rsT), capi.i32p(ciT), ctypes.byref(nN), capi.i32p(rsN), capi.i32p(ciN))
        np.testing.assert_array_equal(h.local[0], rsT[: nT.value + 1])
        np.testing.assert_array_equal(h.local[1], ciT[: rsT[nT.value]])
        np.testing.assert_array_equal(h.local[2], rsN[: nN.value + 1])
    finally:
        h.close()


class _FailingComm(C.Comm):
    rank, size = 0, 2

    def alltoallv_bytes(self, send, scounts, rcounts):
        raise ConnectionError("peer lost")

    def allreduce(self, value, op=C.SUM):
        raise ConnectionError("peer lost")


def test_communicator_failure_is_reported(lib):
    ids = O.box_hex_ids(2, 2, 2, 2)
    with pytest.raises(capi.SpError) as e:
        M.HostHandle(ids.size, ids, _FailingComm(), capi.SIGNED, True)
    assert e.value.status == capi.SP_ERR_COMM


def test_invalid_setup_requests(lib):
    ids = O.box_hex_ids(2, 2, 2, 2)
    comm = C.ThreadComm.create(1)[0]
    for kind, unique in ((capi.UNSIGNED, True), (capi.HALO, True)):
        with pytest.raises(capi.SpError, match="Invalid ogs setup requested"):
            M.HostHandle(ids.size, ids, comm, kind, unique)


# ---------------------------------------------------------------- gloo ranks
def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _gloo_rank(rank, world, port, path, q):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        from oracle import oracle as orc
        orc.load()
        case, ids = load_case(Path(path))
        comm = C.TorchComm()
        h = M.HostHandle(ids[rank].size, ids[rank], comm, capi.SIGNED, False)
        qv = orc.uniform(h.N, case["qseed"] + 1000 * rank)
        ex = M.gloo_exchange()
        res = {}
        for m, name in ((O.Sym, "sym"), (O.NoTrans, "notrans"), (O.Trans, "trans")):
            res[name] = sha(M.gather_scatter(h, orc, qv, 1, capi.ADD, m, ex))
        q.put((rank, res))
        h.close()
    finally:
        dist.destroy_process_group()


def test_gloo_ranks_match_the_reference(lib):
    """Two processes over torch.distributed (gloo): the setup's collectives and the
    pairwise messages go through TorchComm; results equal the reference's."""
    import torch.multiprocessing as mp
    path = GOLDEN / "ogsmr_2r_2x2x2_p2.json"
    case = json.loads(path.read_text())
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_gloo_rank, args=(r, world, port, str(path), q))
             for r in range(world)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=180) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(world):
        for name in ("sym", "notrans", "trans"):
            assert out[r][name] == case["per_rank"][r]["sha256"]["gs_" + name], (r, name)


def test_ranks_without_nodes_or_ids(lib, orc):
    """A rank with no local nodes and one whose ids are all zero take part in every
    collective and get empty operators; the others are unaffected."""
    P = 3
    rng = np.random.default_rng(2)
    ids = [rng.integers(1, 50, 40).astype(np.int64), np.zeros(0, np.int64),
           np.zeros(10, np.int64)]
    ids[0][::3] *= -1
    hh = C.run_threads(P, lambda c: M.HostHandle(ids[c.rank].size, ids[c.rank], c, capi.SIGNED,
                                                 True))
    try:
        assert [(h.N, h.NlocalT, h.NhaloT) for h in hh][1:] == [(0, 0, 0), (10, 0, 0)]
        assert {h.info.NgatherGlobal for h in hh} == {np.unique(np.abs(ids[0])).size}
        _global_check(orc, ids, hh, P, np.int64)
    finally:
        for h in hh:
            h.close()
