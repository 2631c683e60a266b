"""BS0-BS5 kernels on CUDA tensors, through the C ABI.

The functions take the reference kernels' arguments in the reference's order
(``kernel(N, o_a, o_b)`` at BS/BS1/src/bs1Run.cpp:76, ``kernel1(Nblock, N, o_a,
o_tmp)`` / ``kernel2(Nblock, o_tmp, o_norm)`` at BS/BS3/src/bs3Run.cpp:83-84, ...).
Tensors must be contiguous CUDA tensors of the stated dtype; everything runs on
the current torch stream unless ``stream`` is given.
"""
from __future__ import annotations

import torch

from . import capi


def _stream(stream) -> int:
    if stream is None:
        return torch.cuda.current_stream().cuda_stream
    return stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)


def _chk(t: torch.Tensor, dtypes, name: str) -> None:
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if t.dtype not in dtypes:
        raise TypeError(f"{name} has dtype {t.dtype}, expected one of {dtypes}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")


# ---------------------------------------------------------------- BS0
def bs0(N: int, o_a: torch.Tensor, o_b: torch.Tensor, stream=None) -> None:
    """Empty 1x1 launch (BS/BS0/okl/bs0.okl:27-39)."""
    capi.call("sp_bs0", N, o_a.data_ptr(), o_b.data_ptr(), _stream(stream))


class Bs0Graph:
    """``nlaunches`` empty kernels captured once in a CUDA graph."""

    def __init__(self, nlaunches: int, N: int, o_a, o_b, stream=None):
        h = capi.ctypes.c_void_p()
        capi.call("sp_bs0_graph_create", nlaunches, N, o_a.data_ptr(), o_b.data_ptr(),
                  _stream(stream), capi.ctypes.byref(h))
        self._h = h
        self.nlaunches = nlaunches

    def launch(self, stream=None) -> None:
        capi.call("sp_graph_launch", self._h, _stream(stream))

    def __del__(self):
        if getattr(self, "_h", None) and capi._lib is not None:
            capi.status("sp_graph_destroy", self._h)
            self._h = None


# ---------------------------------------------------------------- BS1 / BS2
def bs1(N: int, o_a: torch.Tensor, o_b: torch.Tensor, stream=None) -> None:
    """b[n] = a[n] for n < N (BS/BS1/okl/bs1.okl:27-34)."""
    _chk(o_a, (torch.float64, torch.float32), "o_a")
    _chk(o_b, (o_a.dtype,), "o_b")
    if N > min(o_a.numel(), o_b.numel()):
        raise ValueError("N exceeds the buffers")
    fn = "sp_bs1_copy_f64" if o_a.dtype == torch.float64 else "sp_bs1_copy_f32"
    capi.call(fn, N, o_a.data_ptr(), o_b.data_ptr(), _stream(stream))


def bs2(N: int, alpha: float, o_x: torch.Tensor, beta: float, o_y: torch.Tensor,
        stream=None) -> None:
    """y = alpha*x + beta*y (BS/BS2/okl/bs2.okl:27-36)."""
    _chk(o_x, (torch.float64, torch.float32), "o_x")
    _chk(o_y, (o_x.dtype,), "o_y")
    if N > min(o_x.numel(), o_y.numel()):
        raise ValueError("N exceeds the buffers")
    fn = "sp_bs2_axpy_f64" if o_x.dtype == torch.float64 else "sp_bs2_axpy_f32"
    capi.call(fn, N, float(alpha), o_x.data_ptr(), float(beta), o_y.data_ptr(), _stream(stream))


# ---------------------------------------------------------------- BS3-BS5 (order-exact)
def nblocks_for(N: int, block_size: int) -> int:
    """Nblock = min(ceil(N/bs), bs) (BS/BS3/src/bs3Run.cpp:80-81)."""
    nb = (N + block_size - 1) // block_size
    return max(1, min(nb, block_size))


def bs3_1(Nblocks: int, N: int, o_a, o_tmp, block_size: int = 256, stream=None) -> None:
    _chk(o_a, (torch.float64,), "o_a")
    _chk(o_tmp, (torch.float64,), "o_tmp")
    capi.call("sp_bs3_1_f64", block_size, Nblocks, N, o_a.data_ptr(), o_tmp.data_ptr(),
              _stream(stream))


def bs3_1_fast(Nblocks: int, N: int, o_a, o_tmp, scratch: "ReduceScratch", block_size: int = 256,
               stream=None) -> None:
    """bs3_1 in the integer-pipe form (the drivers' default): o_tmp[0] = sum a*a,
    o_tmp[1:Nblocks] = 0, so that bs3_2 returns o_tmp[0]."""
    _chk(o_a, (torch.float64,), "o_a")
    _chk(o_tmp, (torch.float64,), "o_tmp")
    capi.call("sp_bs3_1_fast_f64", block_size, Nblocks, N, o_a.data_ptr(), o_tmp.data_ptr(),
              scratch.ptr, _stream(stream))


def bs4_1(Nblocks: int, N: int, o_a, o_b, o_tmp, block_size: int = 256, stream=None) -> None:
    for t, n in ((o_a, "o_a"), (o_b, "o_b"), (o_tmp, "o_tmp")):
        _chk(t, (torch.float64,), n)
    capi.call("sp_bs4_1_f64", block_size, Nblocks, N, o_a.data_ptr(), o_b.data_ptr(),
              o_tmp.data_ptr(), _stream(stream))


def bs5_1(Nblocks: int, N: int, o_Ap, alpha: float, o_r, o_tmp, block_size: int = 1024,
          stream=None) -> None:
    for t, n in ((o_Ap, "o_Ap"), (o_r, "o_r"), (o_tmp, "o_tmp")):
        _chk(t, (torch.float64,), n)
    capi.call("sp_bs5_1_f64", block_size, Nblocks, N, o_Ap.data_ptr(), float(alpha),
              o_r.data_ptr(), o_tmp.data_ptr(), _stream(stream))


def bs5_1_fast(Nblocks: int, N: int, o_Ap, alpha: float, o_r, o_tmp, scratch: "ReduceScratch",
               block_size: int = 1024, stream=None) -> None:
    """bs5_1 with r.r on the integer pipe (the drivers' default): r = r + alpha Ap as
    bs5_1 stores it, o_tmp[0] = r.r, o_tmp[1:Nblocks] = 0, so bs5_2 returns o_tmp[0]."""
    for t, n in ((o_Ap, "o_Ap"), (o_r, "o_r"), (o_tmp, "o_tmp")):
        _chk(t, (torch.float64,), n)
    capi.call("sp_bs5_1_fast_f64", block_size, Nblocks, N, o_Ap.data_ptr(), float(alpha),
              o_r.data_ptr(), o_tmp.data_ptr(), scratch.ptr, _stream(stream))


def reduce_finish(Nblocks: int, o_tmp, o_out, block_size: int = 256, stream=None) -> None:
    """bs3_2 / bs4_2 / bs5_2."""
    capi.call("sp_reduce_finish_f64", block_size, Nblocks, o_tmp.data_ptr(), o_out.data_ptr(),
              _stream(stream))


bs3_2 = bs4_2 = bs5_2 = reduce_finish


# ---------------------------------------------------------------- single-launch forms
class ReduceScratch:
    """Zero-filled, 256-byte aligned scratch for the single-launch reductions."""

    def __init__(self, device="cuda"):
        nbytes = int(capi.load().sp_reduce_scratch_bytes())
        self.buf = torch.zeros(nbytes + 256, dtype=torch.uint8, device=device)
        off = (-self.buf.data_ptr()) % 256
        self.ptr = self.buf.data_ptr() + off


def norm2(o_a: torch.Tensor, o_out: torch.Tensor, scratch: ReduceScratch, stream=None) -> None:
    """o_out[0] = sum a*a (FP64 result: the integer-pipe sum of squares for float64
    input, compensated FP32 lanes for float32 input)."""
    _chk(o_a, (torch.float64, torch.float32), "o_a")
    _chk(o_out, (torch.float64,), "o_out")
    fn = "sp_norm2_f64" if o_a.dtype == torch.float64 else "sp_norm2_f32"
    capi.call(fn, o_a.numel(), o_a.data_ptr(), o_out.data_ptr(), scratch.ptr, _stream(stream))


def dot(o_a, o_b, o_out, scratch: ReduceScratch, stream=None) -> None:
    _chk(o_a, (torch.float64, torch.float32), "o_a")
    _chk(o_b, (o_a.dtype,), "o_b")
    _chk(o_out, (torch.float64,), "o_out")
    fn = "sp_dot_f64" if o_a.dtype == torch.float64 else "sp_dot_f32"
    capi.call(fn, o_a.numel(), o_a.data_ptr(), o_b.data_ptr(), o_out.data_ptr(), scratch.ptr,
              _stream(stream))


def cg_update(alpha: float, o_p, o_Ap, o_x, o_r, o_rdotr, scratch: ReduceScratch,
              stream=None) -> None:
    """x += alpha p; r -= alpha Ap; rdotr[0] = r.r (FP64)."""
    _chk(o_p, (torch.float64, torch.float32), "o_p")
    for t, n in ((o_Ap, "o_Ap"), (o_x, "o_x"), (o_r, "o_r")):
        _chk(t, (o_p.dtype,), n)
    _chk(o_rdotr, (torch.float64,), "o_rdotr")
    fn = "sp_cg_update_f64" if o_p.dtype == torch.float64 else "sp_cg_update_f32"
    capi.call(fn, o_p.numel(), float(alpha), o_p.data_ptr(), o_Ap.data_ptr(), o_x.data_ptr(),
              o_r.data_ptr(), o_rdotr.data_ptr(), scratch.ptr, _stream(stream))


def cg_update_ref(alpha: float, o_Ap, o_r, o_rdotr, scratch: ReduceScratch, stream=None) -> None:
    """The reference's BS5 update in one launch: r += alpha Ap; rdotr[0] = r.r (FP64;
    fixed-grid order, compensated FP32 lanes for float32 storage)."""
    _chk(o_Ap, (torch.float64, torch.float32), "o_Ap")
    _chk(o_r, (o_Ap.dtype,), "o_r")
    _chk(o_rdotr, (torch.float64,), "o_rdotr")
    fn = "sp_cg_update_ref_f64" if o_Ap.dtype == torch.float64 else "sp_cg_update_ref_f32"
    capi.call(fn, o_Ap.numel(), float(alpha), o_Ap.data_ptr(), o_r.data_ptr(),
              o_rdotr.data_ptr(), scratch.ptr, _stream(stream))
