"""ctypes binding of ``include/sp_capi.h`` (libspgb300.so).

Every call goes straight to the CUDA library; there is no CPU fallback.  A missing
library raises :class:`SpError` at first use.  Pointers are passed as integers
(``tensor.data_ptr()``), streams as ``torch.cuda.Stream.cuda_stream`` integers
(0 = legacy default stream).
"""
from __future__ import annotations

import ctypes
import re
from ctypes import POINTER, c_double, c_float, c_int32, c_int64, c_size_t, c_uint64, c_void_p
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libspgb300.so"
HEADER = Path(__file__).resolve().parent.parent / "include" / "sp_capi.h"

# status codes (sp_capi.h)
SP_SUCCESS = 0
SP_ERR_INVALID_ARG = 1
SP_ERR_CUDA = 2
SP_ERR_ALLOC = 3
SP_ERR_UNSUPPORTED = 4
SP_ERR_SIZE = 5
SP_ERR_CSR = 6
SP_ERR_TIMEOUT = 7
SP_ERR_DEVICE_CHECK = 8
SP_ERR_COMM = 9

# enums shared with the reference's ogs::Type / Op / Transpose / Kind
FLOAT, DOUBLE, INT32, INT64 = 0, 1, 2, 3
ADD, MUL, MAX, MIN = 0, 1, 2, 3
SYM, NOTRANS, TRANS = 0, 1, 2
UNSIGNED, SIGNED, HALO = 0, 1, 2


class SpError(RuntimeError):
    """A C-ABI call returned a non-success sp_status."""

    def __init__(self, status: int, func: str, message: str):
        self.status = status
        self.func = func
        super().__init__(f"{func} failed with status {status}: {message}")


class OgsInfo(ctypes.Structure):
    _fields_ = [("N", c_int32), ("NrowsT", c_int32), ("NrowsN", c_int32), ("nnzT", c_int32),
                ("nnzN", c_int32), ("NrowBlocksT", c_int32), ("NrowBlocksN", c_int32),
                ("maxRowSize", c_int32), ("NgatherGlobal", c_int64), ("NchunksT", c_int32),
                ("NchunksN", c_int32), ("chunkOrder", c_int32), ("rowOrder", c_int32),
                ("NchunksGS", c_int32), ("gsRowOrder", c_int32), ("NpagesT", c_int32),
                ("pageShift", c_int32), ("waitErrors", c_int32), ("NslabsT", c_int32),
                ("NslabsGS", c_int32), ("slabCodeShift", c_int32), ("slabCodedEntries", c_int64),
                ("slabCodedRows", c_int64)]


class MrInfo(ctypes.Structure):
    _fields_ = [("N", c_int32), ("NlocalP", c_int32), ("NlocalT", c_int32), ("NhaloP", c_int32),
                ("NhaloT", c_int32), ("Nshared", c_int32), ("gather_defined", c_int32),
                ("uploaded", c_int32), ("Ngather", c_int64), ("NgatherGlobal", c_int64)]


class MrSched(ctypes.Structure):
    _fields_ = [("Nsend", c_int32), ("NrowsP", c_int32), ("Nrows", c_int32), ("Ncols", c_int32),
                ("NranksSend", c_int32), ("NranksRecv", c_int32)]


_P = c_void_p
_I32P = POINTER(c_int32)
_I64P = POINTER(c_int64)

# name -> (restype, argtypes); status-returning functions have restype c_int32
SIGNATURES = {
    "sp_last_error_string": (ctypes.c_char_p, []),
    "sp_status_string": (ctypes.c_char_p, [c_int32]),
    "sp_version": (c_int32, []),
    "sp_launch_count": (c_int64, []),
    "sp_launch_count_reset": (None, []),
    "sp_tune_set": (c_int32, [ctypes.c_char_p, c_int64]),
    "sp_tune_get": (c_int32, [ctypes.c_char_p, _I64P]),
    "sp_bs0": (c_int32, [c_int32, _P, _P, _P]),
    "sp_bs0_graph_create": (c_int32, [c_int32, c_int32, _P, _P, _P, POINTER(c_void_p)]),
    "sp_graph_begin": (c_int32, [_P]),
    "sp_graph_end": (c_int32, [_P, POINTER(c_void_p)]),
    "sp_graph_launch": (c_int32, [_P, _P]),
    "sp_graph_destroy": (c_int32, [_P]),
    "sp_bs1_copy_f64": (c_int32, [c_int64, _P, _P, _P]),
    "sp_bs1_copy_f32": (c_int32, [c_int64, _P, _P, _P]),
    "sp_bs2_axpy_f64": (c_int32, [c_int64, c_double, _P, c_double, _P, _P]),
    "sp_bs2_axpy_f32": (c_int32, [c_int64, c_float, _P, c_float, _P, _P]),
    "sp_bs3_1_f64": (c_int32, [c_int32, c_int32, c_int64, _P, _P, _P]),
    "sp_bs3_1_fast_f64": (c_int32, [c_int32, c_int32, c_int64, _P, _P, _P, _P]),
    "sp_bs5_1_fast_f64": (c_int32, [c_int32, c_int32, c_int64, _P, c_double, _P, _P, _P,
                                    _P]),
    "sp_bs4_1_f64": (c_int32, [c_int32, c_int32, c_int64, _P, _P, _P, _P]),
    "sp_bs5_1_f64": (c_int32, [c_int32, c_int32, c_int64, _P, c_double, _P, _P, _P]),
    "sp_reduce_finish_f64": (c_int32, [c_int32, c_int32, _P, _P, _P]),
    "sp_bs4_dot_f64_noalloc": (c_int32, [c_int32, c_int32, c_int64, _P, _P, _P, _P]),
    "sp_reduce_scratch_bytes": (c_size_t, []),
    "sp_norm2_f64": (c_int32, [c_int64, _P, _P, _P, _P]),
    "sp_dot_f64": (c_int32, [c_int64, _P, _P, _P, _P, _P]),
    "sp_norm2_f32": (c_int32, [c_int64, _P, _P, _P, _P]),
    "sp_dot_f32": (c_int32, [c_int64, _P, _P, _P, _P, _P]),
    "sp_cg_update_f64": (c_int32, [c_int64, c_double, _P, _P, _P, _P, _P, _P, _P]),
    "sp_cg_update_f32": (c_int32, [c_int64, c_double, _P, _P, _P, _P, _P, _P, _P]),
    "sp_cg_update_ref_f64": (c_int32, [c_int64, c_double, _P, _P, _P, _P, _P]),
    "sp_cg_update_ref_f32": (c_int32, [c_int64, c_double, _P, _P, _P, _P, _P]),
    "sp_ogs_setup_csr": (c_int32, [c_int32, _I64P, c_int32, c_int32, _I32P, _I32P, _I32P,
                                   _I32P, _I32P, _I32P]),
    "sp_ogs_setup": (c_int32, [c_int32, _I64P, c_int32, c_int32, _P, POINTER(c_void_p)]),
    "sp_ogs_setup_device": (c_int32, [c_int32, _P, c_int32, c_int32, _P, POINTER(c_void_p)]),
    "sp_ogs_plan_create": (c_int32, [c_int32, c_int32, _I32P, _I32P, c_int32, _I32P, _I32P,
                                     _P, POINTER(c_void_p)]),
    "sp_ogs_plan_destroy": (c_int32, [_P]),
    "sp_ogs_plan_info": (c_int32, [_P, POINTER(OgsInfo)]),
    "sp_ogs_plan_csr": (c_int32, [_P, c_int32, _I32P, _I32P]),
    "sp_ogs_block_nnz": (c_int32, []),
    "sp_ogs_gather": (c_int32, [_P, c_int32, c_int32, c_int32, c_int32, _P, _P, _P]),
    "sp_ogs_scatter": (c_int32, [_P, c_int32, c_int32, c_int32, _P, _P, _P]),
    "sp_ogs_gather_scatter": (c_int32, [_P, c_int32, c_int32, c_int32, c_int32, _P, _P]),
    "sp_batch_create": (c_int32, [c_int32, _P, _I64P, _P, _P, _P, _P, _P, _P, _P, _P,
                                  POINTER(c_void_p)]),
    "sp_batch_create_f32": (c_int32, [c_int32, _P, _I64P, _P, _P, _P, _P, _P, _P, _P, _P,
                                      POINTER(c_void_p)]),
    "sp_batch_run": (c_int32, [_P, _P]),
    "sp_batch_destroy": (c_int32, [_P]),
    "sp_mesh_box_hex_ids": (c_int32, [c_int32, c_int32, c_int32, c_int32, c_uint64, _I64P]),
    "sp_mesh_box_hex_ids_device": (c_int32, [c_int32, c_int32, c_int32, c_int32, c_uint64, _P,
                                             _P]),
    "sp_mesh_box_hex_ids_rank": (c_int32, [c_int32, c_int32, c_int32, c_int32, c_uint64, c_int32,
                                           c_int32, _I64P]),
    "sp_ogs_mr_setup": (c_int32, [c_int32, _I64P, c_int32, c_int32, _P, c_int32, _P,
                                  POINTER(c_void_p)]),
    "sp_ogs_mr_destroy": (c_int32, [_P]),
    "sp_ogs_mr_info_get": (c_int32, [_P, POINTER(MrInfo)]),
    "sp_ogs_mr_plan": (c_void_p, [_P, c_int32]),
    "sp_ogs_mr_csr": (c_int32, [_P, c_int32, c_int32, _I32P, _I32P]),
    "sp_ogs_mr_schedule": (c_int32, [_P, c_int32, POINTER(MrSched), _I32P, _I32P, _I32P, _I32P,
                                     _I32P, _I32P, _I32P, _I32P, _I32P]),
    "sp_ogs_mr_exchange_start": (c_int32, [_P, c_int32, c_int32, c_int32, _P, _P, _P]),
    "sp_ogs_mr_exchange_finish": (c_int32, [_P, c_int32, c_int32, c_int32, c_int32, _P, _P, _P]),
}

_STATUS_FREE = {"sp_last_error_string", "sp_status_string", "sp_version", "sp_launch_count",
                "sp_launch_count_reset", "sp_reduce_scratch_bytes", "sp_ogs_block_nnz",
                "sp_ogs_mr_plan"}

_lib: ctypes.CDLL | None = None


def header_functions() -> list[str]:
    """Names of every function declared in include/sp_capi.h."""
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sp_[a-z0-9_]+)\s*\(", text)))


def load() -> ctypes.CDLL:
    """Load libspgb300.so once and attach the signatures."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise SpError(-1, "load", f"{LIB_PATH} is missing: build it with "
                      "`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error() -> str:
    return load().sp_last_error_string().decode(errors="replace")


def call(name: str, *args):
    """Call a status-returning entry point; raise SpError on failure."""
    fn = getattr(load(), name)
    st = fn(*args)
    if name not in _STATUS_FREE and st != SP_SUCCESS:
        raise SpError(st, name, last_error())
    return st


def status(name: str, *args) -> int:
    """Call an entry point and return its status without raising."""
    return getattr(load(), name)(*args)


def tune_set(key: str, value: int) -> None:
    call("sp_tune_set", key.encode(), int(value))


def tune_get(key: str) -> int:
    v = c_int64()
    call("sp_tune_get", key.encode(), ctypes.byref(v))
    return v.value


def i32p(arr):
    """ctypes int32* view of a contiguous numpy int32 array."""
    return arr.ctypes.data_as(_I32P)


def i64p(arr):
    return arr.ctypes.data_as(_I64P)
