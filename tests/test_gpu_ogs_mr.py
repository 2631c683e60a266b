"""Multi-rank gather-scatter on the GPU through the product path: ogs_t with a
communicator of several ranks, run as threads of one process on one GPU
(ThreadComm: each rank has its own stream; the halo rows move by device-to-device
copies between host barriers, no kernel waits on another).  Checked bit for bit
against the reference's own multi-rank results (tests/golden/ogsmr_*.json) and,
for every type, op, k and mode, against the CPU emulation of the same operators
(tests/mr_emul.py)."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest
import torch

import mr_emul as M
from streamparanumal_gb300 import capi
from streamparanumal_gb300 import comm as C
from streamparanumal_gb300 import ogs as O

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = sorted(GOLDEN.glob("ogsmr_*r_*.json"))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def setup_ranks(ids, unique=False, kind=O.Signed):
    P = len(ids)

    def body(c):
        torch.cuda.set_device(0)
        s = torch.cuda.Stream()
        o = O.ogs_t()
        with torch.cuda.stream(s):
            x = ids[c.rank]
            n = x.numel() if isinstance(x, torch.Tensor) else x.size
            o.Setup(n, x, c, kind, O.Pairwise, unique, stream=s)
        s.synchronize()
        return o, s

    return C.run_threads(P, body)


def on_ranks(handles, fn):
    """fn(o, stream, rank) on every rank's thread; returns the results by rank."""
    def body(c):
        torch.cuda.set_device(0)
        o, s = handles[c.rank]
        o.comm = c
        with torch.cuda.stream(s):
            out = fn(o, s, c.rank)
        s.synchronize()
        return out
    return C.run_threads(len(handles), body)


@pytest.mark.parametrize("path", CASES, ids=[p.stem for p in CASES])
def test_gpu_multi_rank_matches_the_reference(cuda, orc, path):
    case = json.loads(path.read_text())
    P = case["ranks"]
    z = np.load(GOLDEN / case["ids_file"])
    ids = [z[f"r{r}"].copy() for r in range(P)]
    hs = setup_ranks(ids)
    for r, (o, _) in enumerate(hs):
        want = case["per_rank"][r]["counts"]
        assert (o.N, o.NlocalP, o.NlocalT, o.NhaloP, o.NhaloT, o.Ngather, o.NgatherGlobal) == (
            want["N"], want["NlocalP"], want["NlocalT"], want["NhaloP"], want["NhaloT"],
            want["Ngather"], want["NgatherGlobal"])
    q = [orc.uniform(o.N, case["qseed"] + 1000 * r) for r, (o, _) in enumerate(hs)]
    g = [orc.uniform(o.NlocalT + o.NhaloT, case["qseed"] + 1000 * r + 1)
         for r, (o, _) in enumerate(hs)]

    for m, name in ((O.Sym, "sym"), (O.NoTrans, "notrans"), (O.Trans, "trans")):
        def gs(o, s, r):
            v = torch.from_numpy(q[r]).cuda()
            o.GatherScatter(v, 1, O.Add, m, stream=s)
            return v.cpu().numpy()

        def ga(o, s, r):
            gv = torch.zeros(g[r].size, dtype=torch.float64, device="cuda")
            o.Gather(gv, torch.from_numpy(q[r]).cuda(), 1, O.Add, m, stream=s)
            return gv.cpu().numpy()

        def sc(o, s, r):
            v = torch.zeros(o.N, dtype=torch.float64, device="cuda")
            o.Scatter(v, torch.from_numpy(g[r]).cuda(), 1, m, stream=s)
            return v.cpu().numpy()

        for fn, key in ((gs, "gs_"), (ga, "gather_"), (sc, "scatter_")):
            res = on_ranks(hs, fn)
            for r in range(P):
                assert sha(res[r]) == case["per_rank"][r]["sha256"][key + name], (key + name, r)

    def gmax(o, s, r):
        v = torch.from_numpy(q[r]).cuda()
        o.GatherScatter(v, 1, O.Max, O.Sym, stream=s)
        return v.cpu().numpy()
    res = on_ranks(hs, gmax)
    for r in range(P):
        assert sha(res[r]) == case["per_rank"][r]["sha256"]["gs_sym_max"]


DTYPES = [(torch.float32, np.float32), (torch.float64, np.float64), (torch.int32, np.int32),
          (torch.int64, np.int64)]


@pytest.mark.parametrize("P,box", [(3, (2, 2, 2, 3)), (4, (2, 2, 1, 2))])
def test_gpu_multi_rank_types_ops_k(cuda, orc, P, box):
    """Own owner draws (unique), every type, op, k in {1, 3} and mode: the GPU result
    equals the CPU emulation of the same operators and schedules bit for bit."""
    nx, ny, nz, p = box
    ids = [O.box_hex_ids(nx, ny, nz, p, 0, size=P, rank=r) for r in range(P)]
    hs = setup_ranks(ids, unique=True)
    views = [M.FromOgs(o) for o, _ in hs]
    rng = np.random.default_rng(7)
    for tt, nt in DTYPES:
        for k in (1, 3):
            vals = [(rng.integers(-5, 6, o.N * k) if nt in (np.int32, np.int64)
                     else rng.standard_normal(o.N * k)).astype(nt) for o, _ in hs]
            for op in (O.Add, O.Mul, O.Max, O.Min):
                for m in (O.Sym, O.NoTrans, O.Trans):
                    def gs(o, s, r):
                        v = torch.from_numpy(vals[r]).cuda()
                        o.GatherScatter(v, k, op, m, stream=s)
                        return v.cpu().numpy()
                    got = on_ranks(hs, gs)
                    ex = M.thread_exchanges(P)
                    want = C.run_threads(P, lambda c: M.gather_scatter(
                        views[c.rank], orc, vals[c.rank], k, op, m, ex[c.rank]))
                    for r in range(P):
                        np.testing.assert_array_equal(got[r], want[r],
                                                      err_msg=f"{nt} k={k} op={op} m={m} r={r}")


def test_gpu_multi_rank_device_ids_and_start_finish(cuda, orc):
    """Ids handed over as CUDA tensors (signs written back), and the Start/Finish
    halves with other work queued between them."""
    P = 2
    ids = [O.box_hex_ids(2, 2, 2, 2, 0, size=P, rank=r, device="cuda") for r in range(P)]
    hs = setup_ranks(ids, unique=True)
    allids = torch.cat([i.cpu() for i in ids]).numpy()
    pos = np.bincount(allids[allids > 0])
    assert set(np.unique(pos[np.unique(np.abs(allids))])) == {1}
    views = [M.FromOgs(o) for o, _ in hs]
    vals = [np.arange(o.N, dtype=np.float64) * (r + 1) for r, (o, _) in enumerate(hs)]

    def gs(o, s, r):
        v = torch.from_numpy(vals[r]).cuda()
        w = torch.ones(1000, device="cuda")
        o.GatherScatterStart(v, 1, O.Add, O.Sym, stream=s)
        w.mul_(2.0)
        o.GatherScatterFinish(v, 1, O.Add, O.Sym, stream=s)
        return v.cpu().numpy()
    got = on_ranks(hs, gs)
    ex = M.thread_exchanges(P)
    want = C.run_threads(P, lambda c: M.gather_scatter(views[c.rank], orc, vals[c.rank], 1,
                                                       O.Add, O.Sym, ex[c.rank]))
    for r in range(P):
        np.testing.assert_array_equal(got[r], want[r])


def test_gpu_ranks_without_nodes_or_ids(cuda, orc):
    P = 3
    rng = np.random.default_rng(2)
    ids = [rng.integers(1, 50, 40).astype(np.int64), np.zeros(0, np.int64),
           np.zeros(10, np.int64)]
    hs = setup_ranks(ids, unique=True)
    views = [M.FromOgs(o) for o, _ in hs]
    vals = [rng.standard_normal(o.N) for o, _ in hs]

    def gs(o, s, r):
        v = torch.from_numpy(vals[r]).cuda()
        o.GatherScatter(v, 1, O.Add, O.Sym, stream=s)
        return v.cpu().numpy()
    got = on_ranks(hs, gs)
    ex = M.thread_exchanges(P)
    want = C.run_threads(P, lambda c: M.gather_scatter(views[c.rank], orc, vals[c.rank], 1,
                                                       O.Add, O.Sym, ex[c.rank]))
    for r in range(P):
        np.testing.assert_array_equal(got[r], want[r])


def _torchcomm_rank(rank, world, port, path, q):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        from oracle import oracle as orc
        orc.load()
        torch.cuda.set_device(0)
        case = json.loads(Path(path).read_text())
        z = np.load(GOLDEN / case["ids_file"])
        ids = z[f"r{rank}"].copy()
        comm = C.TorchComm()
        o = O.ogs_t()
        s = torch.cuda.Stream()
        o.Setup(ids.size, ids, comm, O.Signed, O.Pairwise, False, stream=s)
        v = torch.from_numpy(orc.uniform(o.N, case["qseed"] + 1000 * rank)).cuda()
        res = {}
        for m, name in ((O.Sym, "sym"), (O.NoTrans, "notrans"), (O.Trans, "trans")):
            with torch.cuda.stream(s):
                w = v.clone()
            o.GatherScatter(w, 1, O.Add, m, stream=s)
            s.synchronize()
            res[name] = sha(w.cpu().numpy())
        q.put((rank, res))
    finally:
        dist.destroy_process_group()


def test_gpu_torchcomm_processes_match_the_reference(cuda):
    """Two processes on this GPU over a gloo group: the halo rows travel through
    host memory (TorchComm), as the reference's exchange does without GPU-aware MPI;
    every mode matches the reference's own results bit for bit."""
    import socket
    import torch.multiprocessing as mp
    path = GOLDEN / "ogsmr_2r_2x2x2_p2.json"
    case = json.loads(path.read_text())
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_torchcomm_rank, args=(r, 2, port, str(path), q))
             for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=300) for _ in range(2))
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for r in range(2):
        for name in ("sym", "notrans", "trans"):
            assert out[r][name] == case["per_rank"][r]["sha256"]["gs_" + name], (r, name)


def test_gpu_unsigned_kind(cuda, orc):
    P = 2
    ids = [O.box_hex_ids(2, 2, 1, 2, 0, size=P, rank=r) for r in range(P)]
    hs = setup_ranks(ids, unique=False, kind=O.Unsigned)
    views = [M.FromOgs(o) for o, _ in hs]
    rng = np.random.default_rng(9)
    vals = [rng.integers(-7, 8, o.N).astype(np.int64) for o, _ in hs]
    for m in (O.Sym, O.NoTrans, O.Trans):
        def gs(o, s, r):
            v = torch.from_numpy(vals[r]).cuda()
            o.GatherScatter(v, 1, O.Add, m, stream=s)
            return v.cpu().numpy()
        got = on_ranks(hs, gs)
        ex = M.thread_exchanges(P)
        want = C.run_threads(P, lambda c: M.gather_scatter(views[c.rank], orc, vals[c.rank], 1,
                                                           O.Add, m, ex[c.rank]))
        for r in range(P):
            np.testing.assert_array_equal(got[r], want[r], err_msg=f"mode {m} rank {r}")
