"""CPU emulation of the multi-rank gather-scatter, for the tests.

Restates the data flow of the reference's ogs_t over several ranks
(libs/ogs/ogs.cpp:39-125, 205-301, 394-492; ogsPairwise_t, libs/ogs/ogsPairwise.cpp:
106-156) on numpy arrays with the oracle's one-rank gathers and scatters, driven
by the operators and exchange schedules that sp_ogs_mr_setup built.  The exchange
itself is a callable, so the same emulation runs over gloo ranks or over ranks held
in one process.  Test infrastructure only.
"""
from __future__ import annotations

import ctypes

import numpy as np

from streamparanumal_gb300 import capi
from streamparanumal_gb300.ogs import NoTrans, Sym, Trans, _Sched

MODES = (Sym, NoTrans, Trans)


class HostHandle:
    """The host half of sp_ogs_mr_setup (upload = 0): operators and schedules."""

    def __init__(self, N, ids, comm, kind=capi.SIGNED, unique=True):
        self.sp = comm.as_sp_comm()
        h = ctypes.c_void_p()
        st = capi.status("sp_ogs_mr_setup", N, capi.i64p(ids), kind, int(unique),
                         ctypes.addressof(self.sp), 0, None, ctypes.byref(h))
        if st != capi.SP_SUCCESS:
            raise capi.SpError(st, "sp_ogs_mr_setup", capi.last_error())
        self.h = h
        info = capi.MrInfo()
        capi.call("sp_ogs_mr_info_get", h, ctypes.byref(info))
        self.info = info
        self.N = info.N
        self.NlocalP, self.NlocalT = info.NlocalP, info.NlocalT
        self.NhaloP, self.NhaloT = info.NhaloP, info.NhaloT
        self.local = self._ops(0, info.NlocalT, info.NlocalP)
        self.halo = self._ops(1, info.NhaloT, info.NhaloP)
        self.sched = [_Sched(h, m) for m in MODES]

    def _ops(self, which, rowsT, rowsN):
        out = []
        for trans, rows in ((Trans, rowsT), (NoTrans, rowsN)):
            rs = np.zeros(rows + 1, dtype=np.int32)
            capi.call("sp_ogs_mr_csr", self.h, which, trans, capi.i32p(rs), None)
            ci = np.zeros(max(int(rs[-1]), 1), dtype=np.int32)
            capi.call("sp_ogs_mr_csr", self.h, which, trans, capi.i32p(rs), capi.i32p(ci))
            out += [rs, ci[: int(rs[-1])]]
        return tuple(out)  # rsT, ciT, rsN, ciN

    def close(self):
        if self.h is not None:
            capi.status("sp_ogs_mr_destroy", self.h)
            self.h = None


def _pad(rs, rows):
    """CSR row starts padded with empty rows up to `rows` rows."""
    return np.concatenate([rs, np.full(rows + 1 - rs.size, rs[-1], dtype=np.int32)])


def messages(s, k, send):
    """(peer, send slice) and (peer, receive offset, length) lists of one schedule."""
    sends = [(int(r), send[o * k:(o + c) * k])
             for r, c, o in zip(s.sendRanks, s.sendCounts, s.sendOffsets)]
    recvs = [(int(r), (s.NrowsP + int(o)) * k, int(c) * k)
             for r, c, o in zip(s.recvRanks, s.recvCounts, s.recvOffsets)]
    return sends, recvs


def _halo_exchange(hh, orc, mode, k, op, halo, exchange):
    """Pack, exchange (exchange(sends, recvs, halo) fills halo), reduce."""
    s = hh.sched[mode]
    send = halo.reshape(-1, k)[s.sendIds].ravel() if s.Nsend else halo[:0].copy()
    sends, recvs = messages(s, k, send)
    exchange(sends, recvs, halo)
    return orc.gather(s.postRowStarts, s.postColIds, halo[: s.Ncols * k], k, op)


def _halo_buffer(hh, k, dtype):
    return np.zeros(max(hh.sched[Sym].Ncols, 1) * k, dtype=dtype)


def gather_scatter(hh, orc, v, k, op, trans, exchange):
    lrsT, lciT, lrsN, lciN = hh.local
    hrsT, hciT, hrsN, hciN = hh.halo
    halo = _halo_buffer(hh, k, v.dtype)
    g = orc.gather(hrsN, hciN, v, k, op) if trans == NoTrans else orc.gather(hrsT, hciT, v, k, op)
    halo[: g.size] = g
    out = _halo_exchange(hh, orc, trans, k, op, halo, exchange)
    if trans == Sym:
        v2 = orc.gather_scatter(lrsT, lciT, lrsT, lciT, v, k, op)
    elif trans == NoTrans:
        v2 = orc.gather_scatter(_pad(lrsN, hh.NlocalT), lciN, lrsT, lciT, v, k, op)
    else:
        v2 = orc.gather_scatter(lrsT, lciT, _pad(lrsN, hh.NlocalT), lciN, v, k, op)
    if trans == Trans:
        return orc.scatter(hrsN, hciN, out, v2, k)
    return orc.scatter(hrsT, hciT, out, v2, k)


def gather(hh, orc, v, k, op, trans, exchange):
    """gv = [local rows (NlocalT) | halo rows]; halo rows NhaloT (Sym) or NhaloP."""
    lrsT, lciT, lrsN, lciN = hh.local
    hrsT, hciT, hrsN, hciN = hh.halo
    hrows = hh.NhaloT if trans == Sym else hh.NhaloP
    gv = np.zeros((hh.NlocalT + hrows) * k, dtype=v.dtype)
    loc = orc.gather(lrsN, lciN, v, k, op) if trans == NoTrans else orc.gather(lrsT, lciT, v, k, op)
    gv[: loc.size] = loc
    if trans == Trans:
        halo = _halo_buffer(hh, k, v.dtype)
        g = orc.gather(hrsT, hciT, v, k, op)
        halo[: g.size] = g
        out = _halo_exchange(hh, orc, Trans, k, op, halo, exchange)
        gv[hh.NlocalT * k:] = out[: hh.NhaloP * k]
    else:
        g = orc.gather(hrsN, hciN, v, k, op) if trans == NoTrans else orc.gather(hrsT, hciT, v, k, op)
        gv[hh.NlocalT * k: hh.NlocalT * k + g.size] = g
    return gv


def scatter(hh, orc, v, gv, k, trans, exchange):
    lrsT, lciT, lrsN, lciN = hh.local
    hrsT, hciT, hrsN, hciN = hh.halo
    if trans == Trans:
        v2 = orc.scatter(lrsN, lciN, gv[: hh.NlocalP * k], v, k)
    else:
        v2 = orc.scatter(lrsT, lciT, gv[: hh.NlocalT * k], v, k)
    hg = gv[hh.NlocalT * k:]
    if trans == NoTrans:
        halo = _halo_buffer(hh, k, v.dtype)
        halo[: hh.NhaloP * k] = hg[: hh.NhaloP * k]
        out = _halo_exchange(hh, orc, NoTrans, k, capi.ADD, halo, exchange)
        return orc.scatter(hrsT, hciT, out, v2, k)
    if trans == Trans:
        return orc.scatter(hrsN, hciN, hg[: hh.NhaloP * k], v2, k)
    return orc.scatter(hrsT, hciT, hg[: hh.NhaloT * k], v2, k)


def thread_exchanges(nranks, timeout=120.0):
    """Exchange callables for ranks that run as threads of one process: each call
    posts its messages, waits for every rank, copies its receives and waits again."""
    import threading
    barrier = threading.Barrier(nranks, timeout=timeout)
    posted = [None] * nranks

    def make(r):
        def ex(sends, recvs, halo):
            posted[r] = dict(sends)
            barrier.wait()
            for peer, off, n in recvs:
                msg = posted[peer][r]
                assert msg.size == n, (r, peer, msg.size, n)
                halo[off:off + n] = msg
            barrier.wait()
        return ex

    return [make(r) for r in range(nranks)]


def gloo_exchange(group=None):
    """Exchange callable over torch.distributed (gloo) point-to-point messages."""
    import torch
    import torch.distributed as dist

    def ex(sends, recvs, halo):
        bufs = [(off, torch.empty(n, dtype=torch.from_numpy(halo[:0]).dtype))
                for _, off, n in recvs]
        ops = [dist.P2POp(dist.irecv, b, peer, group=group)
               for (peer, _, _), (_, b) in zip(recvs, bufs)]
        ops += [dist.P2POp(dist.isend, torch.from_numpy(np.ascontiguousarray(m)), peer,
                           group=group) for peer, m in sends]
        if ops:
            for w in dist.batch_isend_irecv(ops):
                w.wait()
        for off, b in bufs:
            halo[off:off + b.numel()] = b.numpy()

    return ex


class FromOgs:
    """The emulation's view of a set-up multi-rank ogs_t (operators and schedules
    read back through the C ABI)."""

    def __init__(self, o):
        self.N = o.N
        self.NlocalP, self.NlocalT, self.NhaloP, self.NhaloT = o.NlocalP, o.NlocalT, o.NhaloP, o.NhaloT
        self.local = o.mr_csr(0, Trans) + o.mr_csr(0, NoTrans)
        self.halo = o.mr_csr(1, Trans) + o.mr_csr(1, NoTrans)
        self.sched = [o.schedule(m) for m in MODES]
