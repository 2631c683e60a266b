"""Batched instances (one persistent launch) and CUDA-graph capture, over the C ABI.

:class:`Batch` mirrors sp_batch_create/run: every instance is a full CG update on
its own vectors plus a BS8 gather+scatter on its own node field and plan.
:class:`Graph` captures whatever the library launches on a stream between
``begin()`` and ``end()`` and replays it with one launch.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import capi


def _stream(stream) -> int:
    if stream is None:
        return torch.cuda.current_stream().cuda_stream
    return stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)


def _ptrs(ts) -> ctypes.Array:
    return (ctypes.c_void_p * len(ts))(*[t.data_ptr() for t in ts])


class Batch:
    def __init__(self, plans, x, r, p, Ap, rdotr, q, alpha, stream=None):
        n = np.ascontiguousarray([t.numel() for t in x], dtype=np.int64)
        h = ctypes.c_void_p()
        self._keep = (plans, x, r, p, Ap, rdotr, q)
        plan_ptrs = (ctypes.c_void_p * len(plans))(*[pl._plan for pl in plans])
        al = (ctypes.c_double * len(alpha))(*map(float, alpha))
        dts = {t.dtype for group in (x, r, p, Ap, q) for t in group}
        if dts == {torch.float64}:
            fn = "sp_batch_create"
        elif dts == {torch.float32}:
            fn = "sp_batch_create_f32"  # FP32 storage, FP64 r.r
        else:
            raise TypeError("batch vectors must be all float64 or all float32")
        if any(t.dtype != torch.float64 for t in rdotr):
            raise TypeError("rdotr must be float64")
        capi.call(fn, len(plans), plan_ptrs, capi.i64p(n), _ptrs(x), _ptrs(r), _ptrs(p),
                  _ptrs(Ap), _ptrs(rdotr), _ptrs(q), al, _stream(stream), ctypes.byref(h))
        self._h = h

    def run(self, stream=None) -> None:
        capi.call("sp_batch_run", self._h, _stream(stream))

    def __del__(self):
        if getattr(self, "_h", None) and capi._lib is not None:
            capi.status("sp_batch_destroy", self._h)
            self._h = None


class Graph:
    """with Graph.capture(stream) as g: <library calls on stream>; then g.launch()."""

    def __init__(self, stream):
        self.stream = stream
        self._h = None

    def begin(self) -> None:
        capi.call("sp_graph_begin", _stream(self.stream))

    def end(self) -> None:
        h = ctypes.c_void_p()
        capi.call("sp_graph_end", _stream(self.stream), ctypes.byref(h))
        self._h = h

    def __enter__(self):
        self.begin()
        return self

    def __exit__(self, exc_type, exc, tb):
        if exc_type is None:
            self.end()
        else:  # close the capture without keeping it
            try:
                self.end()
            except capi.SpError:
                pass
        return False

    def launch(self, stream=None) -> None:
        capi.call("sp_graph_launch", self._h, _stream(stream if stream is not None
                                                       else self.stream))

    def __del__(self):
        if getattr(self, "_h", None) and capi._lib is not None:
            capi.status("sp_graph_destroy", self._h)
            self._h = None
