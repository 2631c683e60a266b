"""The reference's own BS0-BS8 driver sources, unmodified, compile against the
drop-in's C++ headers (streamparanumal_gb300/host/libp) and link against the
drop-in's platform/mesh/ogs implementation and libspgb300.so.

The only mapping is by header name: the drivers include "platform.hpp",
"timer.hpp", "mesh.hpp" (and through them "core.hpp", "ogs.hpp"), which resolve to
the files of the same names in host/libp; STREAM_DIR, which the reference's
makefile passes, is defined on the command line.  Nothing of the drivers is
rewritten.  CPU only: the link is checked here; running the linked drivers needs
a GPU and the reference tree together, which no machine of this build has (the
drop-in's own drivers, bin/BS0 ... bin/BS8, run on the GPU in test_drivers.py).
Skipped when the reference tree is absent."""
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HOST = ROOT / "streamparanumal_gb300" / "host"
REF = Path(os.environ.get("SP_REFERENCE_DIR", "/root/reference"))

pytestmark = pytest.mark.skipif(not (REF / "BS" / "BS1" / "src").is_dir(),
                                reason="reference tree not present")


def cuda_home() -> Path:
    from streamparanumal_gb300 import _build
    return _build._cuda_home()


def compile_one(src: Path, obj: Path, incs: list) -> None:
    cmd = ["g++", "-std=c++17", "-O0", "-c", *[f"-I{i}" for i in incs],
           '-DSTREAM_DIR="' + str(REF) + '"', str(src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, f"{src}:\n{res.stderr[-3000:]}"


@pytest.fixture(scope="module")
def shim_objects(tmp_path_factory, lib):
    out = tmp_path_factory.mktemp("shim")
    incs = [HOST / "libp", ROOT / "include", cuda_home() / "include"]
    srcs = sorted((HOST / "src").glob("*.cpp"))
    objs = [out / (s.stem + ".o") for s in srcs]
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        list(ex.map(lambda so: compile_one(so[0], so[1], incs), zip(srcs, objs)))
    return objs


@pytest.mark.parametrize("bs", range(9))
def test_reference_driver_builds_against_dropin(tmp_path, shim_objects, lib, bs):
    d = REF / "BS" / f"BS{bs}"
    srcs = [d / f"bs{bs}Main.cpp"] + sorted((d / "src").glob("*.cpp"))
    incs = [HOST / "libp", d, ROOT / "include", cuda_home() / "include"]
    objs = [tmp_path / (s.stem + ".o") for s in srcs]
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        list(ex.map(lambda so: compile_one(so[0], so[1], incs), zip(srcs, objs)))
    exe = tmp_path / f"BS{bs}"
    libdir = ROOT / "streamparanumal_gb300" / "lib"
    cmd = ["g++", "-o", str(exe), *map(str, objs), *map(str, shim_objects), f"-L{libdir}",
           "-lspgb300", f"-L{cuda_home() / 'lib64'}", "-lcudart", f"-Wl,-rpath,{libdir}"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-3000:]
    assert exe.exists()
