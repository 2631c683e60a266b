"""The C ABI library loads and exports every entry point of include/*.h; argument
validation returns the documented status before any device work (CPU only)."""
import ctypes
import subprocess

import numpy as np
import pytest

from streamparanumal_gb300 import capi


def test_every_declared_function_is_exported(lib):
    declared = capi.header_functions()
    assert len(declared) >= 30
    out = subprocess.run(["nm", "-D", "--defined-only", str(capi.LIB_PATH)], capture_output=True,
                         text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [f for f in declared if f not in exported]
    assert not missing, f"declared but not exported: {missing}"
    for f in declared:
        assert hasattr(lib, f)
    assert set(declared) == set(capi.SIGNATURES), "ctypes signatures out of sync with header"


def test_build_targets_sm_103a_only():
    from streamparanumal_gb300 import _build
    assert _build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_status_strings(lib):
    assert lib.sp_status_string(0) == b"success"
    assert lib.sp_status_string(capi.SP_ERR_CSR) == b"malformed CSR or ids"
    assert lib.sp_version() == 100
    assert lib.sp_ogs_block_nnz() == 2048
    # a 256-byte header and 32 bytes for each of up to 2048 blocks
    assert lib.sp_reduce_scratch_bytes() == 256 + 32 * 2048


@pytest.mark.parametrize("fn,args", [
    ("sp_bs1_copy_f64", (-1, None, None, None)),
    ("sp_bs2_axpy_f64", (-5, 1.0, None, 1.0, None, None)),
    ("sp_bs3_1_f64", (100, 1, 10, None, None, None)),        # bad block size
    ("sp_bs3_1_f64", (256, 0, 10, None, None, None)),        # nblocks < 1
    ("sp_bs3_1_f64", (256, 257, 10, None, None, None)),      # nblocks > bs
    ("sp_reduce_finish_f64", (1024, 2000, None, None, None)),
    ("sp_norm2_f64", (10, None, None, None, None)),          # null scratch
    ("sp_bs3_1_fast_f64", (100, 1, 10, None, None, None, None)),  # bad block size
    ("sp_bs3_1_fast_f64", (256, 0, 10, None, None, None, None)),  # nblocks < 1
    ("sp_bs3_1_fast_f64", (256, 4, 10, None, None, None, None)),  # null vector/scratch
    ("sp_bs5_1_fast_f64", (100, 1, 10, None, 1.0, None, None, None, None)),  # bad block size
    ("sp_bs5_1_fast_f64", (1024, 1025, 10, None, 1.0, None, None, None, None)),  # nblocks > bs
    ("sp_bs5_1_fast_f64", (1024, 4, 10, None, 1.0, None, None, None, None)),  # null vectors
    ("sp_ogs_gather_scatter", (None, 1, 0, 0, 1, None, None)),  # null plan
    ("sp_ogs_gather", (None, 1, 0, 0, 1, None, None, None)),
    ("sp_ogs_scatter", (None, 1, 0, 1, None, None, None)),
    ("sp_mesh_box_hex_ids", (0, 1, 1, 1, 0, None)),
])
def test_invalid_arguments_are_rejected_without_device_work(lib, fn, args):
    st = capi.status(fn, *args)
    assert st == capi.SP_ERR_INVALID_ARG
    assert capi.last_error()


def test_zero_length_is_a_no_op(lib):
    assert capi.status("sp_bs1_copy_f64", 0, None, None, None) == 0
    assert capi.status("sp_bs2_axpy_f32", 0, 1.0, None, 2.0, None, None) == 0


def _plan_status(N, rs, ci, rsN=None, ciN=None):
    h = ctypes.c_void_p()
    rs = np.ascontiguousarray(rs, dtype=np.int32)
    ci = np.ascontiguousarray(ci if len(ci) else [0], dtype=np.int32)
    if rsN is None:
        return capi.status("sp_ogs_plan_create", N, rs.size - 1, capi.i32p(rs), capi.i32p(ci),
                           rs.size - 1, None, None, None, ctypes.byref(h))
    rsN = np.ascontiguousarray(rsN, dtype=np.int32)
    ciN = np.ascontiguousarray(ciN if len(ciN) else [0], dtype=np.int32)
    return capi.status("sp_ogs_plan_create", N, rs.size - 1, capi.i32p(rs), capi.i32p(ci),
                       rsN.size - 1, capi.i32p(rsN), capi.i32p(ciN), None, ctypes.byref(h))


def test_plan_validation_rejects_malformed_csr(lib):
    # rowStarts[0] != 0
    assert _plan_status(4, [1, 2], [0]) == capi.SP_ERR_CSR
    # not monotone
    assert _plan_status(4, [0, 2, 1], [0, 1]) == capi.SP_ERR_CSR
    # column out of range
    assert _plan_status(4, [0, 1], [4]) == capi.SP_ERR_CSR
    # one column in two rows
    assert _plan_status(4, [0, 1, 2], [3, 3]) == capi.SP_ERR_CSR
    # N member outside its T row
    assert _plan_status(4, [0, 2, 4], [0, 1, 2, 3], [0, 1, 2], [2, 0]) == capi.SP_ERR_CSR
    # NrowsN > NrowsT
    assert _plan_status(4, [0, 1], [0], [0, 0, 0], []) == capi.SP_ERR_CSR


def test_plan_validation_rejects_oversized_group(lib):
    # the reference aborts on multiplicity > 512 (libs/ogs/ogsOperator.cpp:535)
    n = 513
    st = _plan_status(n, [0, n], np.arange(n))
    assert st == capi.SP_ERR_SIZE
    assert "Multiplicity" in capi.last_error()


def test_unique_with_unsigned_kind_is_invalid(lib):
    ids = np.arange(1, 5, dtype=np.int64)
    z = np.zeros(8, dtype=np.int32)
    nT, nN = ctypes.c_int32(), ctypes.c_int32()
    st = capi.status("sp_ogs_setup_csr", 4, capi.i64p(ids), capi.UNSIGNED, 1,
                     ctypes.byref(nT), capi.i32p(z), capi.i32p(z), ctypes.byref(nN),
                     capi.i32p(z), capi.i32p(z))
    assert st == capi.SP_ERR_INVALID_ARG
    assert capi.last_error() == "Invalid ogs setup requested"


KNOB_RANGES = {  # key: (lowest, highest, default), as include/sp_capi.h documents them
    "reduce.prefetch_chunks": (-1, 64, -1), "reduce.rolling": (0, 1, 1),
    "ogs.block_nnz": (256, 2048, 2048), "ogs.order": (0, 2, 1), "ogs.page_shift": (3, 16, 9),
    "ogs.rows": (0, 1, 1), "ogs.ball_shift": (0, 26, 0), "ogs.gs_order": (-1, 2, -1),
    "ogs.gs_page_shift": (3, 16, 8), "ogs.gs_ball_shift": (0, 26, 18),
    "ogs.kernel": (0, 7, 2), "ogs.kernel.gather": (0, 7, 2), "ogs.kernel.scatter": (0, 5, 5),
    "ogs.scatter_pages": (0, 1, 1), "reduce.norm_exact": (0, 1, 0),
    "reduce.norm_ctas": (4, 6, 4), "reduce.norm_roll": (0, 1, 1),
    "ogs.singles": (0, 2, 2), "reduce.rdotr_exact": (0, 1, 0), "ogs.slabs": (0, 1, 0), "ogs.slab_seg_shift": (8, 22, 17),
    "ogs.slab_lane": (0, 16, 0), "ogs.slab_ctas": (0, 4, 0),
    "ogs.slab_load": (0, 3, 0), "ogs.slab_defer": (0, 1, 1),
    "ogs.slab_code_shift": (0, 12, 0), "ogs.slab_row_codes": (0, 1, 0),
    "ogs.kernel.f32": (-1, 7, -1),
    "ogs.kernel.gather.f32": (-1, 7, -1)}


@pytest.mark.parametrize("key", sorted(KNOB_RANGES))
def test_tuning_knobs_ranges_and_defaults(lib, key):
    lo, hi, default = KNOB_RANGES[key]
    start = capi.tune_get(key)
    try:
        for bad in (lo - 1, hi + 1):
            assert capi.status("sp_tune_set", key.encode(), bad) == capi.SP_ERR_INVALID_ARG
        for good in (lo, hi):
            capi.tune_set(key, good)
            assert capi.tune_get(key) == good
    finally:
        capi.tune_set(key, start)
    out = subprocess.run(["python", "-c", "from streamparanumal_gb300 import capi; "
                          f"print(capi.tune_get('{key}'))"], capture_output=True, text=True,
                         check=True).stdout
    assert int(out) == default, "a fresh process starts from the documented default"


def test_unknown_knob_is_rejected(lib):
    assert capi.status("sp_tune_set", b"ogs.no_such_knob", 0) == capi.SP_ERR_INVALID_ARG


@pytest.mark.parametrize("cname,pyname", [("sp_ogs_info", "capi.OgsInfo"),
                                          ("sp_ogs_mr_info", "capi.MrInfo"),
                                          ("sp_ogs_mr_sched", "capi.MrSched"),
                                          ("sp_comm", "comm.SpComm")])
def test_ctypes_structs_match_the_header(tmp_path, cname, pyname):
    """The ctypes mirrors of the ABI's structs have the header's size and field
    offsets (a C program compiled against include/sp_capi.h prints them)."""
    from pathlib import Path
    from streamparanumal_gb300 import comm
    mod, cls = pyname.split(".")
    st = getattr({"capi": capi, "comm": comm}[mod], cls)
    fields = [f[0] for f in st._fields_]
    src = tmp_path / "layout.c"
    src.write_text("#include <stdio.h>\n#include <stddef.h>\n#include \"sp_capi.h\"\n"
                   "int main(void) {\n"
                   f"  printf(\"%zu\\n\", sizeof({cname}));\n" +
                   "".join(f"  printf(\"%zu\\n\", offsetof({cname}, {f}));\n" for f in fields) +
                   "  return 0;\n}\n")
    exe = tmp_path / "layout"
    include = Path(capi.__file__).resolve().parent.parent / "include"
    subprocess.run(["gcc", "-std=c11", f"-I{include}", str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    assert got[0] == ctypes.sizeof(st)
    assert got[1:] == [getattr(st, f).offset for f in fields]
