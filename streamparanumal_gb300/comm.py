"""Communicators for the multi-rank gather-scatter.

The library has no transport of its own (``sp_comm`` in ``include/sp_capi.h``):
setup calls back into a communicator for its all-to-all exchanges and reductions,
and the data exchange of ``ogs_t`` hands each rank's messages to the communicator's
:meth:`Comm.exchange`.  Two communicators are provided:

* :class:`TorchComm` -- one process per rank over a ``torch.distributed`` process
  group (gloo).  Device buffers are staged through host memory, as the reference
  does when its MPI is not GPU-aware (libs/ogs/ogs.cpp:64-80, 97-117);
* :class:`ThreadComm` -- several ranks as threads of one process (each with its
  own stream), exchanging device buffers with device-to-device copies.  The ranks'
  kernels never wait on one another: every wait is a host barrier.

Message matching follows the reference's Pairwise exchange: one message per peer
and direction (ogsPairwise_t::DeviceFinish, libs/ogs/ogsPairwise.cpp:125-156).
"""
from __future__ import annotations

import ctypes
import threading
from ctypes import CFUNCTYPE, POINTER, c_int32, c_int64, c_void_p

import numpy as np
import torch

_ALLTOALLV = CFUNCTYPE(c_int32, c_void_p, c_void_p, POINTER(c_int64), POINTER(c_int64), c_void_p,
                       POINTER(c_int64), POINTER(c_int64), c_int32)
_ALLREDUCE = CFUNCTYPE(c_int32, c_void_p, POINTER(c_int64), c_int32)

SUM, MIN, MAX = 0, 1, 2


class SpComm(ctypes.Structure):
    """ctypes image of ``sp_comm``."""
    _fields_ = [("rank", c_int32), ("size", c_int32), ("ctx", c_void_p),
                ("alltoallv", _ALLTOALLV), ("allreduce_i64", _ALLREDUCE)]


def _bytes_view(ptr: int, nbytes: int) -> np.ndarray:
    if nbytes == 0:
        return np.zeros(0, dtype=np.uint8)
    return np.ctypeslib.as_array(ctypes.cast(ptr, POINTER(ctypes.c_uint8)), shape=(nbytes,))


class Comm:
    """Base communicator: ``rank``, ``size``, byte all-to-all, int64 reduction and
    the pairwise exchange of device buffers."""

    rank: int = 0
    size: int = 1

    # --- to be provided by subclasses
    def alltoallv_bytes(self, send: np.ndarray, scounts: np.ndarray,
                        rcounts: np.ndarray) -> np.ndarray:
        """send/return uint8 arrays; counts in bytes per rank, data packed by rank."""
        raise NotImplementedError

    def allreduce(self, value: int, op: int = SUM) -> int:
        raise NotImplementedError

    def exchange(self, sends, recvs, stream) -> None:
        """sends / recvs: lists of (peer, CUDA tensor view); one message per peer."""
        raise NotImplementedError

    # --- sp_comm binding
    def as_sp_comm(self) -> SpComm:
        """The sp_comm struct for this communicator (callbacks kept alive by self)."""
        def a2a(ctx, send, scount, sdispl, recv, rcount, rdispl, elem):
            try:
                P = self.size
                sc = np.array([scount[i] for i in range(P)], dtype=np.int64) * elem
                sd = np.array([sdispl[i] for i in range(P)], dtype=np.int64) * elem
                rc = np.array([rcount[i] for i in range(P)], dtype=np.int64) * elem
                rd = np.array([rdispl[i] for i in range(P)], dtype=np.int64) * elem
                src = _bytes_view(send or 0, int((sd + sc).max(initial=0)))
                packed = np.concatenate([src[sd[r]:sd[r] + sc[r]] for r in range(P)]) \
                    if sc.sum() else np.zeros(0, dtype=np.uint8)
                got = self.alltoallv_bytes(packed, sc, rc)
                dst = _bytes_view(recv or 0, int((rd + rc).max(initial=0)))
                off = 0
                for r in range(P):
                    dst[rd[r]:rd[r] + rc[r]] = got[off:off + rc[r]]
                    off += int(rc[r])
                return 0
            except Exception as e:  # noqa: BLE001 -- reported as a status
                self.last_error = e
                return 1

        def red(ctx, value, op):
            try:
                value[0] = int(self.allreduce(int(value[0]), int(op)))
                return 0
            except Exception as e:  # noqa: BLE001
                self.last_error = e
                return 1

        self._cb = (_ALLTOALLV(a2a), _ALLREDUCE(red))
        self._sp = SpComm(self.rank, self.size, None, self._cb[0], self._cb[1])
        return self._sp


class TorchComm(Comm):
    """One rank per process over a torch.distributed group (gloo backend).  The
    data exchange stages device buffers through host memory."""

    def __init__(self, group=None):
        import torch.distributed as dist
        self.dist = dist
        self.group = group
        self.rank = dist.get_rank(group)
        self.size = dist.get_world_size(group)

    def _global(self, r: int) -> int:
        return r if self.group is None else self.dist.get_global_rank(self.group, r)

    def alltoallv_bytes(self, send, scounts, rcounts):
        out = torch.empty(int(rcounts.sum()), dtype=torch.uint8)
        inp = torch.from_numpy(np.ascontiguousarray(send)) if send.size else \
            torch.empty(0, dtype=torch.uint8)
        self.dist.all_to_all_single(out, inp, [int(c) for c in rcounts], [int(c) for c in scounts],
                                    group=self.group)
        return out.numpy()

    def allreduce(self, value, op=SUM):
        d = self.dist
        t = torch.tensor([value], dtype=torch.int64)
        d.all_reduce(t, op={SUM: d.ReduceOp.SUM, MIN: d.ReduceOp.MIN, MAX: d.ReduceOp.MAX}[op],
                     group=self.group)
        return int(t.item())

    def exchange(self, sends, recvs, stream):
        d = self.dist
        if stream is not None:
            stream.synchronize()
        host_recv = [(peer, torch.empty(t.shape, dtype=t.dtype)) for peer, t in recvs]
        ops = [d.P2POp(d.irecv, h, self._global(peer), group=self.group) for peer, h in host_recv]
        ops += [d.P2POp(d.isend, t.cpu() if t.is_cuda else t, self._global(peer), group=self.group)
                for peer, t in sends]
        if ops:
            for w in d.batch_isend_irecv(ops):
                w.wait()
        # the uploads go on the caller's stream, ahead of the kernels that reduce them
        with torch.cuda.stream(stream) if stream is not None else _null():
            for (peer, dst), (_, h) in zip(recvs, host_recv):
                dst.copy_(h)


class _ThreadGroup:
    def __init__(self, size: int, timeout: float):
        self.size = size
        self.barrier = threading.Barrier(size, timeout=timeout)
        self.slots = [None] * size


class ThreadComm(Comm):
    """Rank ``rank`` of ``size`` ranks that run as threads of one process."""

    def __init__(self, group: _ThreadGroup, rank: int):
        self.g = group
        self.rank = rank
        self.size = group.size

    @staticmethod
    def create(size: int, timeout: float = 120.0) -> list["ThreadComm"]:
        g = _ThreadGroup(size, timeout)
        return [ThreadComm(g, r) for r in range(size)]

    def _post_and_collect(self, item):
        self.g.slots[self.rank] = item
        self.g.barrier.wait()
        items = list(self.g.slots)
        self.g.barrier.wait()
        return items

    def alltoallv_bytes(self, send, scounts, rcounts):
        offs = np.concatenate([[0], np.cumsum(scounts)])
        items = self._post_and_collect((send, offs))
        parts = []
        for r in range(self.size):
            s, o = items[r]
            parts.append(s[o[self.rank]:o[self.rank + 1]])
        got = np.concatenate(parts) if parts else np.zeros(0, dtype=np.uint8)
        if got.size != int(rcounts.sum()):
            raise RuntimeError("alltoallv: count mismatch")
        return got

    def allreduce(self, value, op=SUM):
        vals = self._post_and_collect(value)
        return {SUM: sum, MIN: min, MAX: max}[op](vals)

    def exchange(self, sends, recvs, stream):
        if stream is not None:
            stream.synchronize()  # the packed send buffer is complete
        self.g.slots[self.rank] = dict(sends)
        self.g.barrier.wait()
        with torch.cuda.stream(stream) if stream is not None else _null():
            for peer, dst in recvs:
                src = self.g.slots[peer].get(self.rank)
                if src is None or src.numel() != dst.numel():
                    raise RuntimeError(f"rank {self.rank}: no matching message from {peer}")
                dst.copy_(src)
        if stream is not None:
            stream.synchronize()
        self.g.barrier.wait()  # every receiver has its copy: send buffers are free


class _null:
    def __enter__(self):
        return None

    def __exit__(self, *a):
        return False


def run_threads(size: int, fn, timeout: float = 300.0):
    """Runs fn(comm) for ranks 0..size-1 as threads; returns the results by rank and
    re-raises the first failure."""
    comms = ThreadComm.create(size)
    out = [None] * size
    err = [None] * size

    def body(r):
        try:
            out[r] = fn(comms[r])
        except BaseException as e:  # noqa: BLE001
            err[r] = e
            comms[r].g.barrier.abort()

    ts = [threading.Thread(target=body, args=(r,)) for r in range(size)]
    for t in ts:
        t.start()
    for t in ts:
        t.join(timeout)
    for e in err:
        if e is not None and not isinstance(e, threading.BrokenBarrierError):
            raise e
    for e in err:
        if e is not None:
            raise e
    return out
