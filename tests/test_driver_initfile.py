"""The driver's init-file parser (oak_io.cpp) against the reference's init-file syntax
(initfile.F90): key = value lines, '#' / '!' comments, 'strings' with '' escapes, one-line
lists, Fortran d exponents, the first definition of a key. Compiled with the host compiler
into a small harness (no GPU)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "oak_gb300", "csrc")


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    out = tmp_path_factory.mktemp("probe") / "initfile_probe"
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", CSRC, os.path.join(HERE, "initfile_probe.cpp"),
                    os.path.join(CSRC, "oak_io.cpp"), "-o", str(out)], check=True)
    return str(out)


def _run(probe, text, tmp_path, *keys):
    f = tmp_path / "t.init"
    f.write_text(text)
    r = subprocess.run([probe, str(f), *keys], capture_output=True, text=True, check=True)
    return r.stdout.strip().splitlines()


def test_reference_syntax(probe, tmp_path):
    text = "\n".join([
        "# comment line",
        "! another comment",
        "Model.variables     = [          'var1',          'var2']",
        "Model.path          = 'tmp-data/'",
        "ErrorSpace.init      = ['(\"Ens\",I3.3,\"/model.nc#var1\")','(\"Ens\",I3.3,\"/m.nc#v\")']",
        "schemetype = 1   # trailing comment",
        "Zones.corrLength.const = [           30e3,             30e3]",
        "Zones.maxLength.const  = [         2000d3,           2.5D-1]  ! comment",
        "quote = 'it''s'",
        "empty = []",
        "schemetype = 0",
        "   indented.key=7",
    ])
    lines = _run(probe, text, tmp_path, "Model.variables", "Model.path", "ErrorSpace.init",
                 "schemetype", "Zones.corrLength.const", "Zones.maxLength.const", "quote",
                 "empty", "indented.key", "absent")
    assert lines == [
        "Model.variables STRS <var1> <var2>",
        "Model.path STRS <tmp-data/>",
        'ErrorSpace.init STRS <("Ens",I3.3,"/model.nc#var1")> <("Ens",I3.3,"/m.nc#v")>',
        "schemetype NUMS 1",
        "Zones.corrLength.const NUMS 30000 30000",
        "Zones.maxLength.const NUMS 2000000 0.25",
        "quote STRS <it's>",
        "empty NUMS",
        "indented.key NUMS 7",
        "absent MISSING",
    ]


@pytest.mark.parametrize("bad", ["key 'no equals'", "k = 'unterminated", "k = [1, 2",
                                 "k = 1 2"])
def test_malformed_lines(probe, tmp_path, bad):
    lines = _run(probe, bad + "\n", tmp_path, "k")
    assert lines[0].startswith("ERROR") and ":1:" in lines[0]


@pytest.fixture(scope="module")
def io_probe(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    out = tmp_path_factory.mktemp("ioprobe") / "io_probe"
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", CSRC, os.path.join(HERE, "io_probe.cpp"),
                    os.path.join(CSRC, "oak_io.cpp"), "-o", str(out)], check=True)
    return str(out)


def _io(io_probe, *args):
    return subprocess.run([io_probe, *map(str, args)], capture_output=True, text=True,
                          check=True).stdout.strip()


def test_fortran_format_file_names(io_probe):
    """loadVectorSpace's file names (assimilation.F90:1214-1220): Fortran I edits."""
    assert _io(io_probe, "fmt", '("Ens",I3.3,"/model.nc#var1")', 7) == "Ens007/model.nc#var1"
    assert _io(io_probe, "fmt", "('S',I3.3,'-obs.nc#var1')", 12) == "S012-obs.nc#var1"
    assert _io(io_probe, "fmt", '("m",I4,".nc#v")', 42) == "m  42.nc#v"
    assert _io(io_probe, "fmt", '("m",I2,".nc")', 123) == "m**.nc"  # Fortran overflow stars
    assert _io(io_probe, "fmt", '("m",F5.2)', 1).startswith("ERROR")
    assert _io(io_probe, "fmt", '"no parentheses"', 1).startswith("ERROR")


def test_replication_of_smaller_files(io_probe):
    """ureadfull_srepmat: a 2-D field replicated along a third dimension, a depth profile
    matched to the third dimension, identical sizes passed through, misfits refused."""
    # file 2 x 3 (values 0..5) onto 2 x 3 x 2: repeated per level
    assert _io(io_probe, "rep", 2, 3, "-", 2, 3, 2) == "0 1 2 3 4 5 0 1 2 3 4 5"
    # file of 3 levels onto 2 x 2 x 3: constant over the horizontal
    assert _io(io_probe, "rep", 3, "-", 2, 2, 3) == "0 0 0 0 1 1 1 1 2 2 2 2"
    # a unit dimension in the file broadcasts
    assert _io(io_probe, "rep", 1, 3, "-", 2, 3) == "0 0 1 1 2 2"
    assert _io(io_probe, "rep", 6, "-", 2, 3) == "0 1 2 3 4 5"
    assert _io(io_probe, "rep", 4, "-", 2, 3).startswith("ERROR")
