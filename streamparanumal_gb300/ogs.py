"""``ogs_t`` over the C ABI, at one rank or over a communicator of several.

Mirrors ``libp::ogs::ogs_t`` (include/ogs.hpp:216-344): ``Setup`` with the same
arguments, then ``Gather`` / ``Scatter`` / ``GatherScatter`` (and their
``Start``/``Finish`` halves) on CUDA tensors.  At one rank there is no halo, so
``*Start`` only validates and ``*Finish`` runs the local operator -- the reference
also queues the local operator in ``*Finish`` (libs/ogs/ogs.cpp:84-125).  With a
communicator of more than one rank (``comm.py``) the handle holds a local and a
halo operator and the flows of libs/ogs/ogs.cpp: the halo rows are gathered and
packed in ``*Start``; ``*Finish`` queues the local operator, exchanges the packed
rows with the peers, reduces what arrived and scatters the halo rows back.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import capi

# re-export the reference's enum names
Float, Double, Int32, Int64 = capi.FLOAT, capi.DOUBLE, capi.INT32, capi.INT64
Add, Mul, Max, Min = capi.ADD, capi.MUL, capi.MAX, capi.MIN
Sym, NoTrans, Trans = capi.SYM, capi.NOTRANS, capi.TRANS
Unsigned, Signed, Halo = capi.UNSIGNED, capi.SIGNED, capi.HALO
Auto, Pairwise, CrystalRouter, AllToAll = 0, 1, 2, 3

_TYPES = {torch.float32: Float, torch.float64: Double, torch.int32: Int32, torch.int64: Int64}


def _stream(stream) -> int:
    if stream is None:
        return torch.cuda.current_stream().cuda_stream
    return stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)


def _vec(t: torch.Tensor, name: str) -> int:
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if t.dtype not in _TYPES:
        raise TypeError(f"{name}: unsupported dtype {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    return _TYPES[t.dtype]


def _stream_obj(stream):
    if stream is None:
        return torch.cuda.current_stream()
    if isinstance(stream, torch.cuda.Stream):
        return stream
    raise TypeError("multi-rank operations take a torch.cuda.Stream (or None)")


class _Sched:
    """Exchange schedule of one transpose mode (sp_ogs_mr_schedule)."""

    def __init__(self, h, mode):
        s = capi.MrSched()
        capi.call("sp_ogs_mr_schedule", h, mode, ctypes.byref(s), None, None, None, None, None,
                  None, None, None, None)
        arr = [np.zeros(max(n, 1), dtype=np.int32) for n in
               (s.NranksSend, s.NranksSend, s.NranksSend, s.NranksRecv, s.NranksRecv,
                s.NranksRecv, s.Nsend, s.Nrows + 1, s.Ncols)]
        capi.call("sp_ogs_mr_schedule", h, mode, ctypes.byref(s), *[capi.i32p(a) for a in arr])
        self.Nsend, self.NrowsP, self.Nrows, self.Ncols = s.Nsend, s.NrowsP, s.Nrows, s.Ncols
        ns, nr = s.NranksSend, s.NranksRecv
        self.sendRanks, self.sendCounts, self.sendOffsets = (a[:ns].copy() for a in arr[0:3])
        self.recvRanks, self.recvCounts, self.recvOffsets = (a[:nr].copy() for a in arr[3:6])
        self.sendIds = arr[6][:s.Nsend].copy()
        self.postRowStarts = arr[7].copy()
        self.postColIds = arr[8][:s.Ncols].copy()


class ogs_t:
    """Gather-scatter handle of one rank (of one or several)."""

    def __init__(self):
        self._plan = None
        self._mr = None
        self.comm = None
        self.N = 0
        self.Ngather = 0
        self.NgatherGlobal = 0
        self.NlocalT = 0
        self.NlocalP = 0
        self.NhaloT = 0
        self.NhaloP = 0
        self.kind = Signed
        self.unique = False

    # ------------------------------------------------------------ setup
    def Setup(self, N: int, ids, comm=None, kind: int = Signed, method: int = Auto,
              unique: bool = False, verbose: bool = False, platform=None, stream=None) -> None:
        """Group the local indices by |ids| (0 = ignored, negative = flagged).

        ``ids`` is a contiguous int64 numpy array (host setup) or CUDA tensor (the
        setup runs on the device, sp_ogs_setup_device; same plan).  With ``unique``
        the signs of ``ids`` are rewritten in place so that every group has one
        positive member, as ogsBase_t::Setup does (libs/ogs/ogsSetup.cpp:145-147).
        ``comm`` is None or a :class:`comm.Comm`: with more than one rank the setup
        is collective over it (host side; device ids are copied to the host and the
        signs written back) and the exchange is Pairwise whatever ``method`` says.
        One rank needs no exchange."""
        self.Free()
        if comm is not None and comm.size > 1:
            self._setup_mr(N, ids, comm, kind, unique, stream)
            if verbose and comm.rank == 0:
                print(f"ogs Setup: {self.NgatherGlobal} gathered nodes over {comm.size} ranks")
            return
        h = ctypes.c_void_p()
        if isinstance(ids, torch.Tensor):
            if not ids.is_cuda or ids.dtype != torch.int64 or not ids.is_contiguous():
                raise TypeError("device ids must be a contiguous CUDA int64 tensor")
            if ids.numel() < N:
                raise ValueError("ids shorter than N")
            capi.call("sp_ogs_setup_device", N, ids.data_ptr(), kind, int(bool(unique)),
                      _stream(stream), ctypes.byref(h))
        else:
            if not isinstance(ids, np.ndarray) or ids.dtype != np.int64 or not ids.flags.c_contiguous:
                raise TypeError("ids must be a contiguous numpy int64 array or CUDA tensor")
            if ids.size < N:
                raise ValueError("ids shorter than N")
            capi.call("sp_ogs_setup", N, capi.i64p(ids), kind, int(bool(unique)), _stream(stream),
                      ctypes.byref(h))
        self._attach(h, kind, unique)
        if verbose:
            print(f"ogs Setup: {self.NgatherGlobal} gathered nodes, {self.info.NrowBlocksT} "
                  f"row blocks")

    def _setup_mr(self, N, ids, comm, kind, unique, stream):
        dev = isinstance(ids, torch.Tensor)
        if dev:
            if ids.dtype != torch.int64 or ids.numel() < N:
                raise TypeError("ids must be an int64 tensor of at least N entries")
            hids = ids[:N].cpu().numpy().copy()
        else:
            if not isinstance(ids, np.ndarray) or ids.dtype != np.int64 or not ids.flags.c_contiguous:
                raise TypeError("ids must be a contiguous numpy int64 array or CUDA tensor")
            if ids.size < N:
                raise ValueError("ids shorter than N")
            hids = ids
        sp = comm.as_sp_comm()
        h = ctypes.c_void_p()
        st = capi.status("sp_ogs_mr_setup", N, capi.i64p(hids), kind, int(bool(unique)),
                         ctypes.addressof(sp), 1, _stream(stream), ctypes.byref(h))
        if st != capi.SP_SUCCESS:
            msg = capi.last_error()
            if getattr(comm, "last_error", None) is not None:
                msg += f" ({comm.last_error!r})"
            raise capi.SpError(st, "sp_ogs_mr_setup", msg)
        if dev and unique:
            ids[:N].copy_(torch.from_numpy(hids))
        self._mr = h
        self.comm = comm
        info = capi.MrInfo()
        capi.call("sp_ogs_mr_info_get", h, ctypes.byref(info))
        self.mr_info = info
        self.N = info.N
        self.NlocalP, self.NlocalT = info.NlocalP, info.NlocalT
        self.NhaloP, self.NhaloT = info.NhaloP, info.NhaloT
        self.Ngather = int(info.Ngather)
        self.NgatherGlobal = int(info.NgatherGlobal)
        self.gather_defined = bool(info.gather_defined)
        self.kind = kind
        self.unique = bool(unique)
        self._local = capi.load().sp_ogs_mr_plan(h, 0)
        self._halo = capi.load().sp_ogs_mr_plan(h, 1)
        self._sched = [_Sched(h, m) for m in (Sym, NoTrans, Trans)]
        self._bufs = {}

    def mr_csr(self, which: int, trans: int = Trans) -> tuple[np.ndarray, np.ndarray]:
        """Host copy of the local (0) or halo (1) operator, T (``Trans``) or N."""
        rows = {(0, Trans): self.NlocalT, (0, NoTrans): self.NlocalP,
                (1, Trans): self.NhaloT, (1, NoTrans): self.NhaloP}[(which, trans)]
        rs = np.zeros(rows + 1, dtype=np.int32)
        capi.call("sp_ogs_mr_csr", self._mr, which, trans, capi.i32p(rs), None)
        ci = np.zeros(max(int(rs[-1]), 1), dtype=np.int32)
        capi.call("sp_ogs_mr_csr", self._mr, which, trans, capi.i32p(rs), capi.i32p(ci))
        return rs, ci[: int(rs[-1])]

    def schedule(self, mode: int) -> _Sched:
        return self._sched[mode]

    def SetupFromCSR(self, N: int, rowStartsT: np.ndarray, colIdsT: np.ndarray,
                     rowStartsN: np.ndarray | None = None, colIdsN: np.ndarray | None = None,
                     stream=None) -> None:
        """Build the handle from explicit T (and optional N) CSR arrays."""
        self.Free()
        rsT = np.ascontiguousarray(rowStartsT, dtype=np.int32)
        ciT = np.ascontiguousarray(colIdsT, dtype=np.int32)
        nT = rsT.size - 1
        h = ctypes.c_void_p()
        if rowStartsN is None:
            capi.call("sp_ogs_plan_create", N, nT, capi.i32p(rsT), capi.i32p(ciT), nT, None, None,
                      _stream(stream), ctypes.byref(h))
        else:
            rsN = np.ascontiguousarray(rowStartsN, dtype=np.int32)
            ciN = np.ascontiguousarray(colIdsN, dtype=np.int32)
            capi.call("sp_ogs_plan_create", N, nT, capi.i32p(rsT), capi.i32p(ciT), rsN.size - 1,
                      capi.i32p(rsN), capi.i32p(ciN), _stream(stream), ctypes.byref(h))
        self._attach(h, Signed, False)

    def plan_info(self) -> capi.OgsInfo:
        """The plan's sp_ogs_info now (waitErrors reads the device: it synchronises)."""
        info = capi.OgsInfo()
        capi.call("sp_ogs_plan_info", self._plan, ctypes.byref(info))
        return info

    def _attach(self, h, kind, unique):
        self._plan = h
        info = capi.OgsInfo()
        capi.call("sp_ogs_plan_info", h, ctypes.byref(info))
        self.info = info
        self.N = info.N
        self.NlocalT = info.NrowsT
        self.NlocalP = info.NrowsN
        self.Ngather = info.NrowsN
        self.NgatherGlobal = int(info.NgatherGlobal)
        self.kind = kind
        self.unique = bool(unique)

    def csr(self, trans: int = Trans) -> tuple[np.ndarray, np.ndarray]:
        """Host copy of the T (``Trans``) or N (``NoTrans``) operator."""
        nrows = self.info.NrowsN if trans == NoTrans else self.info.NrowsT
        nnz = self.info.nnzN if trans == NoTrans else self.info.nnzT
        rs = np.zeros(nrows + 1, dtype=np.int32)
        ci = np.zeros(max(nnz, 1), dtype=np.int32)
        capi.call("sp_ogs_plan_csr", self._plan, trans, capi.i32p(rs), capi.i32p(ci))
        return rs, ci[:nnz]

    def Free(self) -> None:
        if self._plan is not None and capi._lib is not None:
            capi.status("sp_ogs_plan_destroy", self._plan)
        self._plan = None
        if getattr(self, "_mr", None) is not None and capi._lib is not None:
            capi.status("sp_ogs_mr_destroy", self._mr)
        self._mr = None

    def __del__(self):
        self.Free()

    def _need(self):
        if self._plan is None and self._mr is None:
            raise RuntimeError("ogs handle is not set up.")

    def _defined(self):
        if self._mr is not None and not self.gather_defined:
            raise RuntimeError("Gather operation not well-defined.")

    # ------------------------------------------------------------ multi-rank pieces
    def _buffers(self, v: torch.Tensor, k: int):
        key = (v.dtype, k, v.device)
        if key not in self._bufs:
            sym = self._sched[Sym]
            mk = lambda n: torch.empty(max(n, 1) * k, dtype=v.dtype, device=v.device)  # noqa: E731
            self._bufs[key] = (mk(sym.Ncols), mk(sym.Nsend), mk(sym.Nrows))
        return self._bufs[key]

    def _exchange(self, mode, k, halo, send, stream):
        s = self._sched[mode]
        sends = [(int(r), send[o * k:(o + c) * k])
                 for r, c, o in zip(s.sendRanks, s.sendCounts, s.sendOffsets)]
        recvs = [(int(r), halo[(s.NrowsP + o) * k:(s.NrowsP + o + c) * k])
                 for r, c, o in zip(s.recvRanks, s.recvCounts, s.recvOffsets)]
        self.comm.exchange(sends, recvs, stream)

    def _mr_start(self, t, mode, k, halo, send, sh):
        capi.call("sp_ogs_mr_exchange_start", self._mr, t, mode, k, halo.data_ptr(),
                  send.data_ptr(), sh)

    def _mr_finish(self, t, op, mode, k, halo, send, recv, st):
        self._exchange(mode, k, halo, send, st)
        capi.call("sp_ogs_mr_exchange_finish", self._mr, t, op, mode, k, halo.data_ptr(),
                  recv.data_ptr(), st.cuda_stream)

    # ------------------------------------------------------------ operations
    def GatherScatter(self, o_v, k: int, op: int, trans: int, stream=None) -> None:
        self.GatherScatterStart(o_v, k, op, trans, stream)
        self.GatherScatterFinish(o_v, k, op, trans, stream)

    def GatherScatterStart(self, o_v, k, op, trans, stream=None) -> None:
        self._need()
        t = _vec(o_v, "o_v")
        if self._mr is not None:
            if o_v.numel() < self.N * k:
                raise ValueError("o_v shorter than N*k")
            halo, send, _ = self._buffers(o_v, k)
            sh = _stream_obj(stream).cuda_stream
            capi.call("sp_ogs_gather", self._halo, t, op, trans, k, halo.data_ptr(),
                      o_v.data_ptr(), sh)
            self._mr_start(t, trans, k, halo, send, sh)

    def GatherScatterFinish(self, o_v, k, op, trans, stream=None) -> None:
        self._need()
        t = _vec(o_v, "o_v")
        if o_v.numel() < self.N * k:
            raise ValueError("o_v shorter than N*k")
        if self._mr is None:
            capi.call("sp_ogs_gather_scatter", self._plan, t, op, trans, k, o_v.data_ptr(),
                      _stream(stream))
            return
        st = _stream_obj(stream)
        halo, send, recv = self._buffers(o_v, k)
        capi.call("sp_ogs_gather_scatter", self._local, t, op, trans, k, o_v.data_ptr(),
                  st.cuda_stream)
        self._mr_finish(t, op, trans, k, halo, send, recv, st)
        capi.call("sp_ogs_scatter", self._halo, t, trans, k, o_v.data_ptr(), recv.data_ptr(),
                  st.cuda_stream)

    def Gather(self, o_gv, o_v, k: int, op: int, trans: int, stream=None) -> None:
        self.GatherStart(o_gv, o_v, k, op, trans, stream)
        self.GatherFinish(o_gv, o_v, k, op, trans, stream)

    def _gather_rows(self, trans):
        if self._mr is None:
            return self.NlocalP if trans == NoTrans else self.NlocalT
        return self.NlocalT + (self.NhaloT if trans == Sym else self.NhaloP)

    def GatherStart(self, o_gv, o_v, k, op, trans, stream=None) -> None:
        self._need()
        self._defined()
        t = _vec(o_v, "o_v")
        if _vec(o_gv, "o_gv") != t:
            raise TypeError("o_gv and o_v must have the same dtype")
        if self._mr is None:
            return
        if o_gv.numel() < self._gather_rows(trans) * k or o_v.numel() < self.N * k:
            raise ValueError("buffer too short")
        sh = _stream_obj(stream).cuda_stream
        if trans == Trans:  # only the transposed gather talks to the peers
            halo, send, _ = self._buffers(o_v, k)
            capi.call("sp_ogs_gather", self._halo, t, op, Trans, k, halo.data_ptr(),
                      o_v.data_ptr(), sh)
            self._mr_start(t, Trans, k, halo, send, sh)
        else:
            capi.call("sp_ogs_gather", self._halo, t, op, trans, k,
                      o_gv[self.NlocalT * k:].data_ptr(), o_v.data_ptr(), sh)

    def GatherFinish(self, o_gv, o_v, k, op, trans, stream=None) -> None:
        self._need()
        self._defined()
        t = _vec(o_v, "o_v")
        if _vec(o_gv, "o_gv") != t:
            raise TypeError("o_gv and o_v must have the same dtype")
        if o_gv.numel() < self._gather_rows(trans) * k or o_v.numel() < self.N * k:
            raise ValueError("buffer too short")
        if self._mr is None:
            capi.call("sp_ogs_gather", self._plan, t, op, trans, k, o_gv.data_ptr(),
                      o_v.data_ptr(), _stream(stream))
            return
        st = _stream_obj(stream)
        capi.call("sp_ogs_gather", self._local, t, op, trans, k, o_gv.data_ptr(), o_v.data_ptr(),
                  st.cuda_stream)
        if trans == Trans:
            halo, send, recv = self._buffers(o_v, k)
            self._mr_finish(t, op, Trans, k, halo, send, recv, st)
            with torch.cuda.stream(st):
                n = self.NhaloP * k
                o_gv[self.NlocalT * k:self.NlocalT * k + n].copy_(recv[:n])

    def Scatter(self, o_v, o_gv, k: int, trans: int, stream=None) -> None:
        self.ScatterStart(o_v, o_gv, k, trans, stream)
        self.ScatterFinish(o_v, o_gv, k, trans, stream)

    def _scatter_rows(self, trans):
        if self._mr is None:
            return self.NlocalP if trans == Trans else self.NlocalT
        return self.NlocalT + (self.NhaloT if trans == Sym else self.NhaloP)

    def ScatterStart(self, o_v, o_gv, k, trans, stream=None) -> None:
        self._need()
        self._defined()
        t = _vec(o_v, "o_v")
        if _vec(o_gv, "o_gv") != t:
            raise TypeError("o_gv and o_v must have the same dtype")
        if self._mr is None or trans != NoTrans:  # only NoTrans talks to the peers
            return
        if o_gv.numel() < self._scatter_rows(trans) * k or o_v.numel() < self.N * k:
            raise ValueError("buffer too short")
        st = _stream_obj(stream)
        halo, send, _ = self._buffers(o_v, k)
        n = self.NhaloP * k
        with torch.cuda.stream(st):
            halo[:n].copy_(o_gv[self.NlocalT * k:self.NlocalT * k + n])
        self._mr_start(t, NoTrans, k, halo, send, st.cuda_stream)

    def ScatterFinish(self, o_v, o_gv, k, trans, stream=None) -> None:
        self._need()
        self._defined()
        t = _vec(o_v, "o_v")
        if _vec(o_gv, "o_gv") != t:
            raise TypeError("o_gv and o_v must have the same dtype")
        if o_gv.numel() < self._scatter_rows(trans) * k or o_v.numel() < self.N * k:
            raise ValueError("buffer too short")
        if self._mr is None:
            capi.call("sp_ogs_scatter", self._plan, t, trans, k, o_v.data_ptr(), o_gv.data_ptr(),
                      _stream(stream))
            return
        st = _stream_obj(stream)
        capi.call("sp_ogs_scatter", self._local, t, trans, k, o_v.data_ptr(), o_gv.data_ptr(),
                  st.cuda_stream)
        if trans == NoTrans:
            halo, send, recv = self._buffers(o_v, k)
            self._mr_finish(t, Add, NoTrans, k, halo, send, recv, st)
            capi.call("sp_ogs_scatter", self._halo, t, NoTrans, k, o_v.data_ptr(),
                      recv.data_ptr(), st.cuda_stream)
        else:
            capi.call("sp_ogs_scatter", self._halo, t, trans, k, o_v.data_ptr(),
                      o_gv[self.NlocalT * k:].data_ptr(), st.cuda_stream)


def box_hex_ids(nx: int, ny: int, nz: int, p: int, perm_seed: int = 0,
                device=None, stream=None, size: int = 1, rank: int = 0):
    """Global ids of an nx*ny*nz hex box of degree p (see sp_mesh_box_hex_ids): a
    numpy array, or with ``device`` a CUDA tensor filled by the device kernel.
    With ``size`` > 1: the box of rank ``rank`` of ``size`` ranks
    (sp_mesh_box_hex_ids_rank, host)."""
    n = nx * ny * nz * (p + 1) ** 3
    if size > 1:
        ids = np.empty(n, dtype=np.int64)
        capi.call("sp_mesh_box_hex_ids_rank", nx, ny, nz, p, perm_seed, size, rank,
                  capi.i64p(ids))
        return torch.from_numpy(ids).to(device) if device is not None else ids
    if device is not None:
        ids = torch.empty(n, dtype=torch.int64, device=device)
        capi.call("sp_mesh_box_hex_ids_device", nx, ny, nz, p, perm_seed, ids.data_ptr(),
                  _stream(stream))
        return ids
    ids = np.empty(n, dtype=np.int64)
    capi.call("sp_mesh_box_hex_ids", nx, ny, nz, p, perm_seed, capi.i64p(ids))
    return ids
