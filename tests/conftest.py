import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from qstem_gb300 import abi  # noqa: E402

GOLDEN = os.path.join(ROOT, "tests", "golden")
# the reference checkout, for the tests that read its shipped data files
REFERENCE = os.environ.get("QS_REFERENCE_DIR", "")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the GB300 library)")


def params_from_dict(d):
    p = abi.QsParams()
    for name, _ in abi.QsParams._fields_:
        if name == "detectors":
            continue
        # fixtures made before a field existed hold its default
        setattr(p, name, d.get(name, 0))
    for i, (rin, rout, sx, sy) in enumerate(d["detectors"]):
        p.detectors[i].rInside, p.detectors[i].rOutside = rin, rout
        p.detectors[i].shiftX, p.detectors[i].shiftY = sx, sy
    from qstem_gb300 import config
    wl = config.wavelength(float(p.v0))
    import math
    for i in range(p.detectorNum):
        det = p.detectors[i]
        ki = np.float32(math.sin(float(det.rInside) * 0.001) / wl)
        ko = np.float32(math.sin(float(det.rOutside) * 0.001) / wl)
        det.k2Inside, det.k2Outside = np.float32(ki * ki), np.float32(ko * ko)
    return p


class Golden:
    def __init__(self, name):
        self.name = name
        z = np.load(os.path.join(GOLDEN, name + ".npz"))
        self.z = z
        self.params = params_from_dict(json.loads(str(z["params_json"])))
        self.meta = json.loads(str(z["meta_json"]))
        self.case = json.loads(str(z["case_json"]))

    def __getitem__(self, k):
        return self.z[k]

    def __contains__(self, k):
        return k in self.z.files

    def keys(self):
        return self.z.files


GOLDEN_CASES = ["sto64", "sto64q", "sto64bl", "sto64d2", "sto64d2u", "si64cbed", "si64tem", "sto64p2d"]


@pytest.fixture(params=GOLDEN_CASES)
def golden(request):
    return Golden(request.param)


def scan_stack(golden):
    """The transmission the scan of a fixture runs through: every slab's stack
    of an unequally divided cell (with QS_SLAB_STACKS), else the one stack."""
    if "T_slabs" in golden:
        return np.ascontiguousarray(golden["T_slabs"]), True
    return golden["T"], False


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def custom_qsc(tmp_path, split=False):
    """The sto64ft case (doCBED with "Structure Factors: custom") as a .qsc;
    split: every table broken over several lines with comments and blank
    lines between them, as readArray reads on."""
    from tests.golden import make_golden
    from qstem_gb300 import config
    case = Golden("sto64ft").case
    cell, _, _ = make_golden.params_for(case)
    config.write_cfg(cell, str(tmp_path / "cell.cfg"))
    path = str(tmp_path / "run.qsc")
    config.write_qsc(path, cfg_file="cell.cfg", ncell=case["ncell"], nx=case["nx"],
                     resolutionX=case["resolutionX"], v0=case["v0"], slices=case["slices"],
                     sliceThickness=case["sliceThickness"], scan=case["scan"], detectors=case["detectors"],
                     alpha=case["alpha"], mode="CBED", folder="out", saveLevel=case["saveLevel"],
                     custom_sf=make_golden.custom_table("sto"))
    if split:
        lines = []
        for line in open(path).read().split("\n"):
            head, _, vals = line.partition(": ")
            if head in ("k", "Sr", "Ti", "O"):
                v = vals.split()
                lines += [head + ": " + " ".join(v[:7]) + "   % first values",
                          "", "  " + " ".join(v[7:20]), "% a comment line", " ".join(v[20:])]
            else:
                lines.append(line)
        open(path, "w").write("\n".join(lines))
    return path, str(tmp_path / "out")

