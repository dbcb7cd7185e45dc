"""The drop-in adapter (qstem_gb300/adapter/stemlib_gb300.cpp) linked into
the reference's own stem3 program in place of the five hot-path bodies of
stem3/stemlib.cpp (oracle/Makefile, target `adapter`; built by
__graft_entry__.build() where the reference checkout is present).

On the CPU: the program links against libqstem_gpu.so, the five functions
stem3.cpp calls come from the adapter while the reference's own bodies are
still compiled under other names, and a run of an unmodified stem3 input gets
through the reference's readFile and doSTEM to the adapter's first library
call, which without a GPU ends with the library's own error message."""
import os
import shutil
import subprocess

import pytest

from conftest import GOLDEN, ROOT

BIN = os.path.join(ROOT, "oracle", "_ref", "ref_stem3_gpu")
ADAPTER_OBJ = os.path.join(ROOT, "oracle", "_ref", "obj", "stemlib_gb300.o")
MOVED_OBJ = os.path.join(ROOT, "oracle", "_ref", "obj", "stemlib_moved.o")
FUNCS = ["make3DSlices", "initSTEMSlices", "probe", "runMulsSTEM", "collectIntensity"]

pytestmark = pytest.mark.skipif(not os.path.exists(BIN), reason="adapted stem3 not built (needs the reference checkout)")


def defined(obj):
    out = subprocess.run(["nm", "-C", "--defined-only", obj], capture_output=True, text=True, check=True).stdout
    return {line.split(" ", 2)[2].split("(")[0] for line in out.splitlines() if " T " in line}


def test_the_five_bodies_come_from_the_adapter():
    ours, moved = defined(ADAPTER_OBJ), defined(MOVED_OBJ)
    for f in FUNCS:
        assert f in ours, f
        assert f not in moved and "qs_ref_" + f in moved, f
    deps = subprocess.run(["ldd", BIN], capture_output=True, text=True).stdout
    assert "libqstem_gpu.so" in deps and "not found" not in deps.split("libqstem_gpu.so")[1].split("\n")[0]


def test_unmodified_input_reaches_the_library(tmp_path):
    """run.qsc (STEM through two slabs, two detectors, a 5 x 4 raster): the
    reference's readFile and doSTEM run, then make3DSlices asks the library
    for a context; with no usable GPU that call fails with its message."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present: this check is for machines without one")
    except ImportError:
        pass
    for f in os.listdir(os.path.join(GOLDEN, "qsc")):
        shutil.copy(os.path.join(GOLDEN, "qsc", f), tmp_path / f)
    r = subprocess.run([BIN, "run.qsc"], cwd=tmp_path, stdin=subprocess.DEVNULL, capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 1, r.stdout[-2000:] + r.stderr[-2000:]
    assert "qstem_gpu: context:" in r.stderr
    assert "Scan window" in r.stdout  # readFile's summary of the input
