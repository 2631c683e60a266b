"""numpy interface to the CPU restatement (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` as the
checker, and by bench.py's CPU-baseline leg.  The product never calls it.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_double, c_float, c_int, c_int32, c_int64, c_uint64, c_void_p
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "liboracle.so"
_lib = None

_D = POINTER(c_double)
_F = POINTER(c_float)
_I32 = POINTER(c_int32)
_I64 = POINTER(c_int64)

_SIGS = {
    "or_bs1": (None, [c_int64, _D, _D]),
    "or_bs2": (None, [c_int64, c_double, _D, c_double, _D, c_int]),
    "or_bs2_f32": (None, [c_int64, c_float, _F, c_float, _F, c_int]),
    "or_bs3_1": (None, [c_int, c_int, c_int64, _D, _D, c_int]),
    "or_bs4_1": (None, [c_int, c_int, c_int64, _D, _D, _D, c_int]),
    "or_bs5_1": (None, [c_int, c_int, c_int64, _D, c_double, _D, _D, c_int]),
    "or_finish": (None, [c_int, c_int, _D, _D]),
    "or_dot_dd": (c_double, [c_int64, _D, _D]),
    "or_dot_dd_f32": (c_double, [c_int64, _F, _F]),
    "or_cg_update": (c_double, [c_int64, c_double, _D, _D, _D, _D]),
    "or_cg_update_f32": (c_double, [c_int64, c_float, _F, _F, _F, _F]),
    "or_box_hex_ids": (c_int, [c_int, c_int, c_int, c_int, c_uint64, _I64]),
    "or_ogs_setup": (c_int, [c_int32, _I64, c_int, c_int, _I32, _I32, _I32, _I32, _I32, _I32]),
    "or_ogs_gather": (None, [c_int, c_int, c_int32, _I32, _I32, c_int, c_void_p, c_void_p]),
    "or_ogs_scatter": (None, [c_int, c_int32, _I32, _I32, c_int, c_void_p, c_void_p]),
    "or_ogs_gather_scatter": (None, [c_int, c_int, c_int32, _I32, _I32, _I32, _I32, c_int,
                                     c_void_p]),
    "or_fill_uniform": (None, [c_int64, c_uint64, _D]),
}

TYPE_CODE = {np.dtype(np.float32): 0, np.dtype(np.float64): 1, np.dtype(np.int32): 2,
             np.dtype(np.int64): 3}


def load():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            from streamparanumal_gb300 import _build
            _build.build_oracle()
        lib = ctypes.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _d(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_D)


def _f(a):
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(_F)


def _i32(a):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_I32)


def _i64(a):
    assert a.dtype == np.int64 and a.flags.c_contiguous
    return a.ctypes.data_as(_I64)


# ---------------------------------------------------------------- inputs
def uniform(n: int, seed: int) -> np.ndarray:
    """Seeded uniform[-1,1) FP64 (SplitMix64 stream)."""
    x = np.empty(n, dtype=np.float64)
    load().or_fill_uniform(n, seed, _d(x))
    return x


# ---------------------------------------------------------------- BS1..BS5
def bs2(alpha, x, beta, y, fmad=1):
    y = y.copy()
    if y.dtype == np.float64:
        load().or_bs2(y.size, alpha, _d(x), beta, _d(y), fmad)
    else:
        load().or_bs2_f32(y.size, np.float32(alpha), _f(x), np.float32(beta), _f(y), fmad)
    return y


def bs3(a, bs=256, nblocks=None, fmad=1):
    """Returns (partials, result) of bs3_1 + bs3_2."""
    n = a.size
    nb = nblocks or max(1, min((n + bs - 1) // bs, bs))
    part = np.zeros(nb, dtype=np.float64)
    load().or_bs3_1(bs, nb, n, _d(a), _d(part), fmad)
    out = np.zeros(1, dtype=np.float64)
    load().or_finish(bs, nb, _d(part), _d(out))
    return part, out[0]


def bs4(a, b, bs=256, nblocks=None, fmad=1):
    n = a.size
    nb = nblocks or max(1, min((n + bs - 1) // bs, bs))
    part = np.zeros(nb, dtype=np.float64)
    load().or_bs4_1(bs, nb, n, _d(a), _d(b), _d(part), fmad)
    out = np.zeros(1, dtype=np.float64)
    load().or_finish(bs, nb, _d(part), _d(out))
    return part, out[0]


def bs5(Ap, alpha, r, bs=1024, nblocks=None, fmad=1):
    """Returns (updated r, partials, result)."""
    n = r.size
    nb = nblocks or max(1, min((n + bs - 1) // bs, bs))
    r = r.copy()
    part = np.zeros(nb, dtype=np.float64)
    load().or_bs5_1(bs, nb, n, _d(Ap), alpha, _d(r), _d(part), fmad)
    out = np.zeros(1, dtype=np.float64)
    load().or_finish(bs, nb, _d(part), _d(out))
    return r, part, out[0]


def finish(partial, bs):
    out = np.zeros(1, dtype=np.float64)
    load().or_finish(bs, partial.size, _d(partial), _d(out))
    return out[0]


def dot_dd(a, b):
    if a.dtype == np.float32:
        return load().or_dot_dd_f32(a.size, _f(a), _f(b))
    return load().or_dot_dd(a.size, _d(a), _d(b))


def cg_update(alpha, p, Ap, x, r):
    """Returns (x, r, r.r) with x, r updated in fma form."""
    x = x.copy()
    r = r.copy()
    if x.dtype == np.float64:
        rr = load().or_cg_update(x.size, alpha, _d(p), _d(Ap), _d(x), _d(r))
    else:
        rr = load().or_cg_update_f32(x.size, np.float32(alpha), _f(p), _f(Ap), _f(x), _f(r))
    return x, r, rr


# ---------------------------------------------------------------- mesh / ogs
def box_hex_ids(nx, ny, nz, p, perm_seed=0) -> np.ndarray:
    ids = np.empty(nx * ny * nz * (p + 1) ** 3, dtype=np.int64)
    if load().or_box_hex_ids(nx, ny, nz, p, perm_seed, _i64(ids)):
        raise ValueError("bad box arguments")
    return ids


def ogs_setup(ids: np.ndarray, kind=1, unique=False):
    """Returns dict(rsT, ciT, rsN, ciN) and modifies ids in place when unique."""
    N = ids.size
    rsT = np.zeros(N + 1, dtype=np.int32)
    ciT = np.zeros(max(N, 1), dtype=np.int32)
    rsN = np.zeros(N + 1, dtype=np.int32)
    ciN = np.zeros(max(N, 1), dtype=np.int32)
    nT = c_int32()
    nN = c_int32()
    rc = load().or_ogs_setup(N, _i64(ids), kind, int(unique), ctypes.byref(nT), _i32(rsT),
                             _i32(ciT), ctypes.byref(nN), _i32(rsN), _i32(ciN))
    if rc:
        raise ValueError("Invalid ogs setup requested")
    rsT = rsT[: nT.value + 1].copy()
    rsN = rsN[: nN.value + 1].copy()
    return dict(rsT=rsT, ciT=ciT[: rsT[-1]].copy(), rsN=rsN, ciN=ciN[: rsN[-1]].copy())


def gather(rs, ci, v, k=1, op=0, nrows=None):
    nrows = rs.size - 1 if nrows is None else nrows
    gv = np.zeros(nrows * k, dtype=v.dtype)
    load().or_ogs_gather(TYPE_CODE[v.dtype], op, nrows, _i32(rs), _i32(ci), k,
                         gv.ctypes.data_as(c_void_p), v.ctypes.data_as(c_void_p))
    return gv


def scatter(rs, ci, gv, v, k=1, nrows=None):
    """Returns a copy of v with the scatter applied."""
    nrows = rs.size - 1 if nrows is None else nrows
    v = v.copy()
    load().or_ogs_scatter(TYPE_CODE[v.dtype], nrows, _i32(rs), _i32(ci), k,
                          v.ctypes.data_as(c_void_p), gv.ctypes.data_as(c_void_p))
    return v


def gather_scatter(grs, gci, srs, sci, v, k=1, op=0, nrows=None):
    nrows = grs.size - 1 if nrows is None else nrows
    v = v.copy()
    load().or_ogs_gather_scatter(TYPE_CODE[v.dtype], op, nrows, _i32(grs), _i32(gci), _i32(srs),
                                 _i32(sci), k, v.ctypes.data_as(c_void_p))
    return v
