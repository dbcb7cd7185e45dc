"""The C restatement (oracle/) against fixtures produced by the reference
itself (tests/golden/make_golden.py).  On the build machine the agreement is
bit-exact; the tolerances below only absorb last-bit differences of another
machine's libm (cos/sin/exp of the host the tests run on)."""
import numpy as np
import pytest

from conftest import Golden, rel_l2, scan_stack
from oracle import oracle
from qstem_gb300 import abi

TOL = 1e-5  # relative; bit-exact where the C library is the one the fixtures were made with


@pytest.fixture(scope="module", autouse=True)
def _build():
    oracle.build()


def lut_B(golden, Z, charged):
    """Debye-Waller factor the reference's LUT was built with: that of the
    element's first contributing atom (its static LUT cache is per element,
    stem3/stemlib.cpp:1417); the harness builds tables of elements without
    such atoms itself with B = 0."""
    a = golden["atoms"]
    sel = a[(a["Znum"] == Z) & ((a["q"] != 0) if charged else True)]
    if golden.params.tds or len(sel) == 0:
        return 0.0
    return float(sel["dw"][0])


def test_lut(golden):
    p = golden.params
    for k in golden.keys():
        if not (k.startswith("lut_") or k.startswith("lutq_")):
            continue
        Z = int(k.split("_")[1])
        charged = k.startswith("lutq_")
        mine, nzsub = oracle.lut(p, Z, lut_B(golden, Z, charged), charged=charged)
        ref = golden[k]
        assert mine.shape == ref.shape
        assert nzsub == int(golden["nzsub"])
        assert np.abs(mine - ref).max() <= TOL * np.abs(ref).max(), k


def test_lut2d(golden):
    """getAtomPotential2D's tables (the 2-D potential, potential3D: no)."""
    keys = [k for k in golden.keys() if k.startswith("lut2d_")]
    if not keys:
        pytest.skip("not a 2-D potential case")
    for k in keys:
        Z = int(k.split("_")[1])
        mine = oracle.lut2d(golden.params, Z, lut_B(golden, Z, False))
        ref = golden[k]
        assert mine.shape == ref.shape
        assert np.abs(mine - ref).max() <= TOL * np.abs(ref).max(), k


def test_potential(golden):
    V = oracle.potential(golden.params, golden["atoms"])
    ref = golden["V"]
    assert np.abs(V - ref).max() <= TOL * np.abs(ref).max()
    assert np.all(V[..., 1] == 0)


def test_slab_potentials(golden):
    if "V_slabs" not in golden:
        pytest.skip("not an unequally divided cell")
    p = golden.params
    for k in range(p.cellDiv):
        V = oracle.potential(p, golden["atoms"], slab=k)
        ref = golden["V_slabs"][k]
        assert np.abs(V - ref).max() <= TOL * np.abs(ref).max(), k
        T = oracle.transmission(p, V)
        assert np.abs(T - golden["T_slabs"][k]).max() <= TOL * 1.0, k


def test_transmission(golden):
    T = oracle.transmission(golden.params, golden["V"])
    ref = golden["T"]
    assert np.abs(T - ref).max() <= TOL * max(1.0, np.abs(ref).max())


def test_probe(golden):
    pr = oracle.probe(golden.params)
    ref = golden["probe"]
    assert np.abs(pr - ref).max() <= TOL * np.abs(ref).max()


def test_stem_detectors_diffpats_waves(golden):
    if "det" not in golden:
        pytest.skip("case does not run the scan")
    p = golden.params
    T, slabs = scan_stack(golden)
    det, dps, ews = oracle.stem(p, T, golden["probe"], diffpats=True, exit_waves=True, slab_stacks=slabs)
    ref = golden["det"]
    assert det.shape == ref.shape
    assert rel_l2(det, ref) <= TOL
    for k in golden.keys():
        if k.startswith("diffpat_") or k.startswith("wave_"):
            ix, iy = map(int, k.split("_")[1:])
            pos = ix * p.scanYN + iy
            mine = dps[pos] if k.startswith("diffpat_") else ews[pos]
            assert rel_l2(mine, golden[k]) <= TOL, k


def test_params_match_readfile(golden):
    """qstem_gb300.config.make_params reproduces readFile's derived fields."""
    p, m = golden.params, golden.meta
    for key in ("nx", "ny", "potNx", "potNy", "slices", "scanXN", "scanYN", "outputInterval",
                "nonPeriod", "nonPeriodZ", "centerSlices", "bandlimittrans"):
        assert getattr(p, key) == int(m[key]), key
    for key in ("resolutionX", "sliceThickness", "potOffsetX", "potOffsetY", "potSizeX", "potSizeY",
                "scanXStart", "scanXStop", "scanYStop", "v0", "alpha", "Cs", "df0", "electronScale", "ax", "by",
                "czOffset"):
        assert np.float32(getattr(p, key)) == np.float32(float(m[key])), key
    for i in range(p.detectorNum):
        vals = [float(v) for v in m["det%d" % i].split()]
        assert np.float32(p.detectors[i].k2Inside) == np.float32(vals[2])
        assert np.float32(p.detectors[i].k2Outside) == np.float32(vals[3])


def test_atoms_match_readunitcell(golden):
    """qstem_gb300.config.replicate reproduces readUnitCell's atom list bit for bit."""
    import sys, os
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    import make_golden
    cell, atoms, _ = make_golden.params_for(golden.case)
    assert np.array_equal(atoms.view(np.uint8), golden["atoms"].view(np.uint8))


def test_thickness_slots(golden):
    """tCount + 1 slots over all slices of all slabs (stem3/stemlib.cpp:2591),
    and the reference's detector arrays have that many."""
    p = golden.params
    assert p.thickness_count() == (p.slices * p.cellDiv // p.outputInterval) + 1
    if "det" in golden:
        assert golden["det"].shape[0] == p.thickness_count()


def cbed_probe_offset(p):
    """doCBED's probe position (stem3/stem3.cpp:2096-2100): the scan start
    minus the potential offset, in the reference's float fields."""
    return (float(np.float32(p.scanXStart) - np.float32(p.potOffsetX)),
            float(np.float32(p.scanYStart) - np.float32(p.potOffsetY)))


def test_cbed_pattern(golden):
    if "cbed_diffpat" not in golden:
        pytest.skip("not a CBED run")
    p = golden.params
    pr = oracle.probe(p, *cbed_probe_offset(p))
    _, _, dp = oracle.run_position(p, golden["T"], 0, 0, pr)
    assert rel_l2(dp, golden["cbed_diffpat"]) <= TOL


def test_tem_exit_wave(golden):
    if "exit_wave" not in golden:
        pytest.skip("not a TEM run")
    p = golden.params
    plane = np.zeros((p.nx, p.ny, 2), np.float32)
    plane[..., 0] = 1.0
    w, _, _ = oracle.run_position(p, golden["T"], 0, 0, plane)
    assert rel_l2(w, golden["exit_wave"]) <= TOL


def test_custom_scattering_factors():
    """make3DSlicesFT with a custom table ("Structure Factors: custom"; the
    fixture is doCBED's run of it): the restatement's potential and
    transmission against the reference's (bit-exact here), and the CBED
    pattern through the restated stack."""
    g = Golden("sto64ft")
    p = g.params
    V = oracle.potential_ft(p, g["atoms"], g["sf_k"], g["sf_Z"], g["sf_f"])
    assert np.abs(V - g["V"]).max() <= TOL * np.abs(g["V"]).max()
    assert np.all(V[..., 1] == 0)
    T = oracle.transmission(p, V)
    assert np.abs(T - g["T"]).max() <= TOL
    pr = oracle.probe(p, *cbed_probe_offset(p))
    _, _, dp = oracle.run_position(p, T, 0, 0, pr)
    assert rel_l2(dp, g["cbed_diffpat"]) <= TOL
