"""The BS0-BS8 drivers keep the reference's command line and output rows
(BS/BSx/src/bsxSettings.cpp, bsxRun.cpp)."""
import re
import subprocess

import pytest

from streamparanumal_gb300 import _build

ROW_VEC = r"-?\d+ [-+.\deE]+ [-+.\deE]+ +[-+.\d]+"
ROW_OGS = (r"BS{w} = \[(\d+), (\d+), [-+.\deE]+, [-+.\deE]+, +[-+.\d]+, +[-+.\d]+\]; % {t} "
           r"\[N, DOFs, elapsed, DOFs/\(ranks\*s\), avg BW \(GB/s\), avg GFLOPs\]")


@pytest.fixture(scope="module")
def bsdir(lib):
    return _build.build_host().parent


def run(bsdir, name, *args, check=True):
    res = subprocess.run([str(bsdir / name), *map(str, args)], capture_output=True, text=True,
                         timeout=600)
    if check:
        assert res.returncode == 0, res.stdout + res.stderr
    return res


def test_usage_lists_reference_keys(bsdir):
    out = run(bsdir, "BS8", "-h").stdout
    for key in ("-m --mode", "-nx --dimx", "-ny --dimy", "-nz --dimz", "-p --degree",
                "-e --elements"):
        assert key in out
    out = run(bsdir, "BS1", "-h").stdout
    for key in ("-b --bytes", "-bmin --bmin", "-bmax --bmax", "-s --bstep"):
        assert key in out
    out = run(bsdir, "BS0", "-h").stdout
    for key in ("-n --Nlaunch", "-nmin --NlaunchMin", "-nmax --NlaunchMax", "-s --step"):
        assert key in out


def test_bad_options_abort(bsdir):
    res = run(bsdir, "BS1", "-zz", "3", check=False)
    assert res.returncode == 1 and "Unrecognized setting" in res.stderr
    res = run(bsdir, "BS8", "-p", "16", check=False)
    assert res.returncode == 1 and "not valid" in res.stderr
    res = run(bsdir, "BS3", "-m", "Serial", check=False)
    assert res.returncode == 1 and "CUDA mode only" in res.stderr


@pytest.mark.gpu
def test_bs0_rows(cuda, bsdir):
    out = run(bsdir, "BS0", "-n", 50).stdout
    assert re.fullmatch(r"BS0 = \[50 [-+.\deE]+ [-+.\deE]+\]; %Launch Latency \[Nlaunches, "
                        r"time per launch, elapsed\]\n", out), out
    out = run(bsdir, "BS0", "-nmin", 1, "-nmax", 3, "-g", "TRUE").stdout
    assert out.startswith("%Launch Latency [Nlaunches, time per launch, elapsed]\nBS0 = [\n1 ")


@pytest.mark.gpu
@pytest.mark.parametrize("which,title", [(1, "Copy"), (2, "AXPY"), (3, "Norm"), (4, "Dot"),
                                         (5, "CG Update")])
@pytest.mark.parametrize("extra", [[], ["-fp", "FP32"], ["-cg", "TRUE"],
                                   ["-fp", "FP32", "-cg", "TRUE"], ["-ex", "TRUE"]])
def test_bs1_to_bs5_rows(cuda, bsdir, which, title, extra):
    out = run(bsdir, f"BS{which}", "-b", 1 << 22, *extra).stdout
    assert re.fullmatch(rf"BS{which} = \[{ROW_VEC}\]; %{title} \[DOFs, elapsed, DOFs/s, BW "
                        r"\(GB/s\)\]\n", out), out
    out = run(bsdir, f"BS{which}", "-bmin", 1 << 20, "-bmax", 3 << 20, "-s", 1 << 20,
              *extra).stdout
    # sweep block: header, "BSx = [", entries separated by ";\n", and "]; %title [...]"
    # right after the last entry (bs1Run.cpp:86-90: ";" only while N < Nmax)
    m = re.fullmatch(rf"%{title} \[DOFs, elapsed, DOFs/s, BW \(GB/s\)\]\nBS{which} = \[\n"
                     rf"((?:{ROW_VEC};\n)*{ROW_VEC};?\n?)\]; %{title} \[DOFs, elapsed, DOFs/s, "
                     r"BW \(GB/s\)\]\n", out)
    assert m, out
    assert len(re.findall(ROW_VEC, m.group(1))) == 3


@pytest.mark.gpu
@pytest.mark.parametrize("which,title", [(6, "Gather"), (7, "Scatter"), (8, "GatherScatter")])
@pytest.mark.parametrize("extra", [[], ["-fp", "FP32"], ["-ps", "7"]])
def test_bs6_to_bs8_rows(cuda, bsdir, which, title, extra):
    out = run(bsdir, f"BS{which}", "-nx", 6, "-ny", 5, "-nz", 4, "-p", 3, *extra).stdout
    m = re.fullmatch(ROW_OGS.format(w=which, t=title) + r" \n", out)
    assert m, out
    assert int(m.group(1)) == 3
    assert int(m.group(2)) == (6 * 3 + 1) * (5 * 3 + 1) * (4 * 3 + 1)


@pytest.mark.gpu
def test_bs8_applies_the_tuning_table(cuda, bsdir, tmp_path):
    out = run(bsdir, "BS8", "-nx", 3, "-ny", 3, "-nz", 3, "-p", 3, "-v", "TRUE").stdout
    assert "tuning: p3 " in out
    out = run(bsdir, "BS8", "-nx", 3, "-ny", 3, "-nz", 3, "-p", 3, "-ps", 5, "-v", "TRUE").stdout
    assert "tuning: p3_perm " in out
    out = run(bsdir, "BS8", "-nx", 3, "-ny", 3, "-nz", 3, "-p", 3, "-t", "NONE", "-v",
              "TRUE").stdout
    assert "tuning:" not in out
    table = tmp_path / "t.txt"
    table.write_text("p3 ogs.order=0 ogs.rows=0 ogs.kernel=0\n")
    out = run(bsdir, "BS8", "-nx", 3, "-ny", 3, "-nz", 3, "-p", 3, "-t", table, "-v",
              "TRUE").stdout
    assert "tuning: p3 ogs.order=0 ogs.rows=0 ogs.kernel=0" in out
    res = run(bsdir, "BS8", "-p", 3, "-t", tmp_path / "missing.txt", check=False)
    assert res.returncode == 1 and "Cannot read tuning file" in res.stderr
