"""In-tree build of the native libraries.

* ``streamparanumal_gb300/lib/libspgb300.so`` -- the CUDA kernels (sm_103a) and the
  C ABI declared in ``include/sp_capi.h``.  Compiled with nvcc, one translation unit
  per process, static cudart so the library loads without extra search paths.
* ``oracle/liboracle.so`` -- the CPU restatement used by the tests as the checker
  (built by :func:`build_oracle`; never linked into the product).

Objects are rebuilt only when a source or header is newer than the library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "lib"
LIB = LIBDIR / "libspgb300.so"
BUILD = ROOT / "_build"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build step failed ({res.returncode}): {' '.join(cmd)}\n"
                           f"{res.stdout}\n{res.stderr}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def sources() -> tuple[list[Path], list[Path], list[Path]]:
    cu = sorted(CSRC.glob("*.cu"))
    cpp = sorted(CSRC.glob("*.cpp"))
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "sp_capi.h"]
    return cu, cpp, headers


def build_library(force: bool = False, verbose: bool = False) -> Path:
    """Compile every CUDA/C++ source of the package into libspgb300.so."""
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    cu, cpp, headers = sources()
    if not force and not _stale(LIB, cu + cpp + headers + [Path(__file__)]):
        return LIB
    obj_dir = BUILD / "obj"
    obj_dir.mkdir(parents=True, exist_ok=True)
    LIBDIR.mkdir(parents=True, exist_ok=True)
    inc = ["-I", str(ROOT / "include"), "-I", str(CSRC)]
    jobs = []
    for src in cu:
        obj = obj_dir / (src.stem + ".cu.o")
        jobs.append([nvcc, *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-fopenmp", *inc, "-c", str(src), "-o", str(obj)])
    for src in cpp:
        obj = obj_dir / (src.stem + ".cpp.o")
        jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", *inc,
                     "-I", str(cuda / "include"), "-c", str(src), "-o", str(obj)])
    workers = max(1, min(len(jobs), os.cpu_count() or 4))
    with ThreadPoolExecutor(max_workers=workers) as ex:
        list(ex.map(_run, jobs))
    objs = [j[-1] for j in jobs]
    tmp = LIB.with_suffix(".so.tmp")
    _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *objs,
          "-Xcompiler", "-fopenmp", "-lgomp"])
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


HOST = PKG / "host"
BINDIR = PKG / "bin"
BS_EXE = BINDIR / "spbs"


def build_host(force: bool = False) -> Path:
    """Compile the C++ mirror of the reference's platform_t / ogs_t / mesh_t
    (host/libp, host/src) and the BS0-BS8 drivers (host/bs) into bin/spbs, linked
    against libspgb300.so, with BS0 ... BS8 as links to it."""
    cuda = _cuda_home()
    srcs = sorted((HOST / "src").glob("*.cpp")) + sorted((HOST / "bs").glob("*.cpp"))
    hdrs = sorted((HOST / "libp").glob("*.hpp")) + sorted((HOST / "bs").glob("*.hpp")) + \
        [ROOT / "include" / "sp_capi.h"]
    BINDIR.mkdir(parents=True, exist_ok=True)
    if force or _stale(BS_EXE, srcs + hdrs + [LIB]):
        obj_dir = BUILD / "host"
        obj_dir.mkdir(parents=True, exist_ok=True)
        inc = ["-I", str(ROOT / "include"), "-I", str(HOST / "libp"), "-I", str(HOST / "bs"),
               "-I", str(cuda / "include")]
        jobs = [["g++", "-O2", "-std=c++17", "-Wall", *inc, "-c", str(src), "-o",
                 str(obj_dir / (src.parent.name + "_" + src.stem + ".o"))] for src in srcs]
        with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
            list(ex.map(_run, jobs))
        tmp = BS_EXE.with_suffix(".tmp")
        _run(["g++", "-o", str(tmp), *[j[-1] for j in jobs], "-L", str(LIBDIR), "-lspgb300",
              "-Wl,-rpath,$ORIGIN/../lib", "-L", str(cuda / "lib64"), "-lcudart",
              f"-Wl,-rpath,{cuda / 'lib64'}"])
        os.replace(tmp, BS_EXE)
    for i in range(9):
        link = BINDIR / f"BS{i}"
        if link.is_symlink() or link.exists():
            link.unlink()
        link.symlink_to(BS_EXE.name)
    return BS_EXE


ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "liboracle.so"


def build_oracle(force: bool = False) -> Path:
    """Compile the CPU restatement (test checker only) with gcc + OpenMP.

    ``-ffp-contract=off`` keeps every multiply-add exactly as written: the oracle
    states its fused multiply-adds with explicit ``fma()`` calls."""
    srcs = sorted(ORACLE_DIR.glob("*.c"))
    hdrs = sorted(ORACLE_DIR.glob("*.h"))
    if not srcs:
        raise RuntimeError("oracle sources missing")
    if not force and not _stale(ORACLE_LIB, srcs + hdrs):
        return ORACLE_LIB
    tmp = ORACLE_LIB.with_suffix(".so.tmp")
    _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
          "-o", str(tmp), *map(str, srcs), "-lm"])
    os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


if __name__ == "__main__":
    build_library(force=True, verbose=True)
    build_host(force=True)
    build_oracle(force=True)
