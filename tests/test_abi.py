"""The C-ABI library builds for sm_103a, loads, and exports every entry point
include/qstem_gpu.h declares (no GPU needed: nothing is launched)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT
from qstem_gb300 import abi, lib

HEADER = os.path.join(ROOT, "include", "qstem_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(qs_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def L():
    from qstem_gb300 import build
    build.build()
    return lib.load()


def test_exports_every_declared_symbol(L):
    names = declared_functions()
    assert len(names) >= 10
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(lib.EXPORTS)


def test_abi_version(L):
    assert L.qs_abi_version() == 3


def test_struct_layouts():
    assert ctypes.sizeof(abi.QsAtom) == 28
    assert abi.ATOM_DTYPE.itemsize == 28
    assert ctypes.sizeof(abi.QsDetector) == 24
    # field order of qs_params as declared in the header
    text = open(HEADER).read()
    body = text[text.index("typedef struct qs_params"):text.index("} qs_params;")]
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    names = []
    for decl in re.findall(r"(?:int|float|qs_detector)\s+([^;]+);", body):
        for n in decl.split(","):
            names.append(n.strip().split("[")[0])
    assert names == [f[0] for f in abi.QsParams._fields_]


def test_params_finalize_and_thickness(L):
    from qstem_gb300 import config
    p = config.make_params(nx=64, resolutionX=0.1, v0=200, slices=20, sliceThickness=2, ax=20, by=20, c=40,
                           scan=(5, 9, 4, 5, 9, 4), detectors=[(70, 200, "HAADF")], outputInterval=7)
    k_in, k_out = p.detectors[0].k2Inside, p.detectors[0].k2Outside
    p.detectors[0].k2Inside = 0
    assert L.qs_params_finalize(ctypes.byref(p)) == 0
    assert np.float32(p.detectors[0].k2Inside) == np.float32(k_in)
    assert np.float32(p.detectors[0].k2Outside) == np.float32(k_out)
    assert L.qs_thickness_count(ctypes.byref(p)) == 20 // 7 + 1


def test_struct_sizes_and_offsets_match_the_c_compiler(tmp_path):
    """ctypes mirrors of the header's structs against gcc's own layout."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = {"qs_atom": abi.QsAtom, "qs_detector": abi.QsDetector, "qs_params": abi.QsParams,
               "qs_batch": abi.QsBatch, "qs_stats": abi.QsStats, "qs_ctf": abi.QsCtf,
               "qs_cbed_job": abi.QsCbedJob, "qs_cbed_report": abi.QsCbedReport}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "qstem_gpu.h"', "int main(void) {"]
    for cname, ct in structs.items():
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for f in ct._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, f[0], cname, f[0]))
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, ct in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(ct), cname
        for f in ct._fields_:
            assert got[(cname, f[0])] == getattr(ct, f[0]).offset, (cname, f[0])


def test_noalloc_refuses_bad_arguments_before_any_device_work(L):
    """qs_multislice_run_noalloc checks its arguments on the host before it
    touches a device: non-positive energy, sampling or slice thickness, and
    a batch that takes its positions from an empty scan raster, come back as
    QS_ERR_ARG (no arithmetic on a zero raster size)."""
    from qstem_gb300 import config
    p0 = config.make_params(nx=64, resolutionX=0.1, v0=200, slices=4, sliceThickness=2, ax=20, by=20, c=8,
                            scan=(5, 9, 4, 5, 9, 4), detectors=[(70, 200, "HAADF")])
    dummy = ctypes.c_void_p(16)  # never dereferenced: the checks fail first
    for field, value in (("v0", 0.0), ("v0", -200.0), ("resolutionX", 0.0), ("sliceThickness", 0.0),
                         ("scanYN", 0), ("scanXN", 0)):
        p = p0.copy()
        setattr(p, field, value)
        b = abi.QsBatch(4, None, None, None, None)
        rc = L.qs_multislice_run_noalloc(None, ctypes.byref(p), dummy, dummy, ctypes.byref(b), dummy, None, None)
        assert rc == abi.QS_ERR_ARG, (field, value, rc)
        assert L.qs_last_error()
