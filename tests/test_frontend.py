"""Host front end: .img format and the input writers (no GPU)."""
import os

import numpy as np

from conftest import REFERENCE
from qstem_gb300 import config, imageio


def test_img_roundtrip(tmp_path):
    rng = np.random.default_rng(0)
    re_ = rng.standard_normal((12, 7)).astype(np.float32)
    c = (rng.standard_normal((5, 9)) + 1j * rng.standard_normal((5, 9))).astype(np.complex64)
    f1, f2 = str(tmp_path / "r.img"), str(tmp_path / "c.img")
    imageio.write_img(f1, re_, t=3.5, dx=0.1, dy=0.2, params=[1.0, 2.5], comment="STEM image")
    imageio.write_img(f2, c, comment="Wavefunction")
    a, b = imageio.read_img(f1), imageio.read_img(f2)
    assert np.array_equal(a.data, re_) and a.comment == "STEM image" and list(a.params) == [1.0, 2.5]
    assert a.t == 3.5 and abs(a.dx - 0.1) < 1e-15
    assert np.array_equal(b.data, c) and b.complex


def test_reference_img_fixtures():
    """The three .img files the reference ships read with the documented
    header and the expected magnitudes (tests/data of the reference)."""
    d = os.path.join(REFERENCE, "tests", "data")
    if not REFERENCE or not os.path.isdir(d):
        import pytest
        pytest.skip("reference checkout not given (QS_REFERENCE_DIR)")
    det = imageio.read_img(os.path.join(d, "detector1_2.img"))
    assert det.data.shape == (20, 20) and det.comment == "detector1" and len(det.params) == 402
    w = imageio.read_img(os.path.join(d, "mulswav_16_2.img"))
    assert w.data.shape == (400, 400) and w.complex
    assert abs(np.mean(np.abs(w.data) ** 2) - 0.9711) < 1e-3


def test_wavelength():
    assert abs(config.wavelength(200) - 0.025079) < 1e-6
    assert abs(config.wavelength(300) - 0.019687) < 1e-6


def test_scan_offsets_match_oracle():
    from oracle import oracle
    import ctypes
    oracle.build()
    p = config.make_params(nx=64, resolutionX=0.0763, v0=200, slices=4, sliceThickness=2, ax=20, by=20, c=8,
                           scan=(7.81, 11.715, 16, 7.81, 11.715, 16), detectors=[(70, 200, "H")])
    px, py, dx, dy = config.scan_offsets(p)
    L = oracle.lib()
    for i in range(p.scanXN * p.scanYN):
        a, b = ctypes.c_int(), ctypes.c_int()
        L.qso_scan_offsets(ctypes.byref(p), i // p.scanYN, i % p.scanYN, ctypes.byref(a), ctypes.byref(b))
        assert (px[i], py[i]) == (a.value, b.value)
    assert p.potNx == 64 + 51  # 3.905/0.0763 -> 51 pixels of scan range
