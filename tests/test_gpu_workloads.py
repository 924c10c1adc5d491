"""Parity and accuracy at the benchmark workloads themselves (full size):

* the PEC cavity (FP64, 60x60x120, 1220 steps): the CUDA path against the CPU oracle within
  1e-10 relative L2 on WP, Z and the final fields;
* the reference's own tests/test_001 golden vectors (FP32, 50x50x150, 5184 steps) with
  the tolerances of that test, and against the reference's full run of the same case;
* the lossy cavity (128x128x256, both beam runs): FP32 against the FP64 CUDA path (itself
  checked against the oracle at 1e-10 on the smaller cases) -- WP within 1e-4.
"""

import numpy as np
import pytest
import torch

import cases as C
from oracle_runner import load_golden, rel_l2, run_oracle_case
from product_runner import run_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")


def test_cavity_60x60x120_fp64_matches_oracle(tmp_path):
    case = C.WORKLOADS["cavity_60x60x120"]
    got = run_case("cavity_60x60x120", case=case, tmpdir=tmp_path)
    ref = run_oracle_case("cavity_60x60x120", case=case)
    assert int(got["Nt"]) == int(ref["Nt"])
    np.testing.assert_array_equal(got["s"], ref["s"])
    np.testing.assert_array_equal(got["f"], ref["f"])
    for k in ("WP", "Z", "E", "H", "WP_3d"):
        assert rel_l2(got[k], ref[k]) < 1e-10, (k, rel_l2(got[k], ref[k]))
    for k, r in (("WPx", "WP"), ("WPy", "WP"), ("Zx", "Z"), ("Zy", "Z")):
        e = np.linalg.norm(got[k] - ref[k]) / max(np.linalg.norm(ref[k]), 1e-3 * np.linalg.norm(ref[r]))
        assert e < 1e-10, (k, e)


def test_reference_test001_goldens_on_gpu(tmp_path):
    import wakis_gb300 as wg
    z = load_golden("test001")
    b = z["bounds"]
    x = np.linspace(b[0], b[1], 51)
    y = np.linspace(b[2], b[3], 51)
    zz = np.linspace(b[4], b[5], 151)
    tol = 1e-3 * min(np.diff(x).min(), np.diff(y).min(), np.diff(zz).min())
    mask = C.test001_boxes_corner_rule(x, y, zz, tol)
    grid = wg.GridFIT3D(*b, 50, 50, 150, stl_solids={"cavity": mask}, stl_materials={"cavity": "vacuum"}, verbose=0)
    wake = wg.WakeSolver(wakelength=1.0, q=1e-9, sigmaz=18.5e-3, beta=1.0, xsource=0.0, ysource=0.0, xtest=0.0,
                         ytest=0.0, save=False, skip_cells=12, verbose=0, results_folder=str(tmp_path))
    solver = wg.SolverFIT3D(grid, wake, bc_low=["pec"] * 3, bc_high=["pec"] * 3, use_stl=True, bg="pec",
                            dtype=np.float32, verbose=0)
    solver.wakesolve(wakelength=1.0)
    assert solver.Nt == int(z["Nt"])
    # the reference test's own assertions (tests/test_001_pec_cubic_cavity.py:153-177)
    assert np.allclose(wake.WP[::50], z["WP_samples"], rtol=50e-6, atol=50e-6)
    assert np.cumsum(np.abs(wake.WP))[-1] == pytest.approx(float(z["WP_cumsum"]), 0.1)
    for f in (np.abs, np.real, np.imag):
        assert np.allclose(f(wake.Z)[::20], f(z["Z_samples"]), rtol=50e-5, atol=50e-5)
    assert np.cumsum(np.abs(wake.Z))[-1] == pytest.approx(float(z["Z_cumsum"]), 0.1)
    # and the reference's full run of the same case
    np.testing.assert_array_equal(wake.s, z["s"])
    assert rel_l2(wake.WP, z["WP"]) < 1e-4
    assert rel_l2(wake.Z, z["Z"]) < 1e-4


@pytest.mark.parametrize("name", ["lossy_cavity_128x128x256", "lossy_cavity_128x128x256_offset"])
def test_lossy_cavity_fp32_against_fp64(name, tmp_path):
    """FP32 fields against FP64 fields at the same time step.  An FP32 solver rounds dt
    to float32 (as the reference does); run at the FP64 CFL step instead, the wake's time
    index int(.../dt) flips for some (s, z) pairs and moves WP near the bunch by ~1e-3
    -- a sampling effect of the post-processor, not of the field precision -- so the
    FP64 run is given the FP32 run's dt."""
    case = C.WORKLOADS[name]
    r32 = run_case(name, case=case, tmpdir=tmp_path, dtype=np.float32)
    r64 = run_case(name, case=dict(case, dtype="float64"), tmpdir=tmp_path, dtype=np.float64, dt=float(r32["dt"]))
    assert int(r32["Nt"]) == int(r64["Nt"])
    np.testing.assert_array_equal(r32["s"], r64["s"])
    assert rel_l2(r32["WP"], r64["WP"]) < 1e-4
    assert rel_l2(r32["Z"], r64["Z"]) < 1e-4


def test_lossy_cavity_coded_equals_dense(tmp_path, monkeypatch):
    """The full lossy-cavity run (128x128x256, lossy walls, PML, 4452 steps) with coded
    coefficients gives the dense run's wake bit for bit."""
    case = C.WORKLOADS["lossy_cavity_128x128x256"]
    out = {}
    for codes in ("1", "0"):
        monkeypatch.setenv("WAKIS_GB300_CODES", codes)
        out[codes] = run_case("lossy_cavity_128x128x256", case=case, tmpdir=tmp_path, dtype=np.float32)
    for k in ("WP", "Z", "WPx", "WPy", "E", "H"):
        np.testing.assert_array_equal(out["1"][k], out["0"][k], err_msg=k)
