"""``ogs_t`` at one rank, over the C ABI.

Mirrors ``libp::ogs::ogs_t`` (include/ogs.hpp:216-344): ``Setup`` with the same
arguments, then ``Gather`` / ``Scatter`` / ``GatherScatter`` (and their
``Start``/``Finish`` halves) on CUDA tensors.  At one rank there is no halo, so
``*Start`` only validates and ``*Finish`` runs the local operator -- the reference
also queues the local operator in ``*Finish`` (libs/ogs/ogs.cpp:84-125).
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


class ogs_t:
    """Gather-scatter handle of one rank."""

    def __init__(self):
        self._plan = None
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
        ``comm``/``method`` are accepted for signature compatibility; one rank needs
        no exchange."""
        self.Free()
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

    def __del__(self):
        self.Free()

    def _need(self):
        if self._plan is None:
            raise RuntimeError("ogs handle is not set up.")

    # ------------------------------------------------------------ operations
    def GatherScatter(self, o_v, k: int, op: int, trans: int, stream=None) -> None:
        self.GatherScatterStart(o_v, k, op, trans, stream)
        self.GatherScatterFinish(o_v, k, op, trans, stream)

    def GatherScatterStart(self, o_v, k, op, trans, stream=None) -> None:
        self._need()
        _vec(o_v, "o_v")

    def GatherScatterFinish(self, o_v, k, op, trans, stream=None) -> None:
        self._need()
        t = _vec(o_v, "o_v")
        if o_v.numel() < self.N * k:
            raise ValueError("o_v shorter than N*k")
        capi.call("sp_ogs_gather_scatter", self._plan, t, op, trans, k, o_v.data_ptr(),
                  _stream(stream))

    def Gather(self, o_gv, o_v, k: int, op: int, trans: int, stream=None) -> None:
        self.GatherStart(o_gv, o_v, k, op, trans, stream)
        self.GatherFinish(o_gv, o_v, k, op, trans, stream)

    def GatherStart(self, o_gv, o_v, k, op, trans, stream=None) -> None:
        self._need()
        _vec(o_gv, "o_gv")
        _vec(o_v, "o_v")

    def GatherFinish(self, o_gv, o_v, k, op, trans, stream=None) -> None:
        self._need()
        t = _vec(o_v, "o_v")
        if _vec(o_gv, "o_gv") != t:
            raise TypeError("o_gv and o_v must have the same dtype")
        rows = self.NlocalP if trans == NoTrans else self.NlocalT
        if o_gv.numel() < rows * k or o_v.numel() < self.N * k:
            raise ValueError("buffer too short")
        capi.call("sp_ogs_gather", self._plan, t, op, trans, k, o_gv.data_ptr(), o_v.data_ptr(),
                  _stream(stream))

    def Scatter(self, o_v, o_gv, k: int, trans: int, stream=None) -> None:
        self.ScatterStart(o_v, o_gv, k, trans, stream)
        self.ScatterFinish(o_v, o_gv, k, trans, stream)

    def ScatterStart(self, o_v, o_gv, k, trans, stream=None) -> None:
        self._need()
        _vec(o_v, "o_v")
        _vec(o_gv, "o_gv")

    def ScatterFinish(self, o_v, o_gv, k, trans, stream=None) -> None:
        self._need()
        t = _vec(o_v, "o_v")
        if _vec(o_gv, "o_gv") != t:
            raise TypeError("o_gv and o_v must have the same dtype")
        rows = self.NlocalP if trans == Trans else self.NlocalT
        if o_gv.numel() < rows * k or o_v.numel() < self.N * k:
            raise ValueError("buffer too short")
        capi.call("sp_ogs_scatter", self._plan, t, trans, k, o_v.data_ptr(), o_gv.data_ptr(),
                  _stream(stream))


def box_hex_ids(nx: int, ny: int, nz: int, p: int, perm_seed: int = 0,
                device=None, stream=None):
    """Global ids of an nx*ny*nz hex box of degree p (see sp_mesh_box_hex_ids): a
    numpy array, or with ``device`` a CUDA tensor filled by the device kernel."""
    n = nx * ny * nz * (p + 1) ** 3
    if device is not None:
        ids = torch.empty(n, dtype=torch.int64, device=device)
        capi.call("sp_mesh_box_hex_ids_device", nx, ny, nz, p, perm_seed, ids.data_ptr(),
                  _stream(stream))
        return ids
    ids = np.empty(n, dtype=np.int64)
    capi.call("sp_mesh_box_hex_ids", nx, ny, nz, p, perm_seed, capi.i64p(ids))
    return ids
