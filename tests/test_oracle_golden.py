"""Pins the CPU oracle against the reference: fixtures generated by running the reference
itself (tests/golden/make_golden.py) and the golden vectors of the reference's
tests/test_001_pec_cubic_cavity.py."""

import numpy as np
import pytest

import cases as C
from oracle_runner import load_golden, rel_l2, run_oracle_case

TOL = {"float64": 1e-12, "float32": 2e-5}


@pytest.mark.parametrize("name", list(C.CASES))
def test_oracle_matches_reference(name):
    case = C.CASES[name]
    g = load_golden(name)
    o = run_oracle_case(name)
    tol = TOL[case["dtype"]]
    for k, v in g.items():
        if k == "Nt":
            assert int(o[k]) == int(v)
        elif k == "dt":
            assert o[k] == v
        elif k in ("s", "f"):
            np.testing.assert_array_equal(o[k], v)
        else:
            assert np.shape(o[k]) == np.shape(v), k
            scale = max(float(np.linalg.norm(np.asarray(v, dtype=np.complex128))), 1e-300)
            if k in ("WPx", "WPy", "Zx", "Zy"):
                # transverse wakes of symmetric cases are ~0: compare on the scale of WP / Z
                ref = g["WP"] if k.startswith("WP") else g["Z"]
                scale = max(scale, 1e-3 * np.linalg.norm(ref))
            err = float(np.linalg.norm(np.asarray(o[k], dtype=np.complex128) - v)) / scale
            assert err <= tol, f"{name}:{k} rel err {err:.3e} > {tol}"


def test_test001_goldens_are_reproduced_by_reference_fixture():
    """The reference run with the analytic corner-rule mask (fixture) passes the
    reference test's own tolerances -- the mask stands in for the STL voxelisation."""
    z = load_golden("test001")
    assert np.allclose(z["WP"][::50], z["WP_samples"], rtol=5e-5, atol=5e-5)
    for f in (np.abs, np.real, np.imag):
        assert np.allclose(f(z["Z"])[::20], f(z["Z_samples"]), rtol=5e-4, atol=5e-4)
    assert np.cumsum(np.abs(z["WP"]))[-1] == pytest.approx(float(z["WP_cumsum"]), 0.1)
    assert np.cumsum(np.abs(z["Z"]))[-1] == pytest.approx(float(z["Z_cumsum"]), 0.1)


@pytest.mark.slow
def test_oracle_test001_goldens():
    """Full test_001 run (50x50x150, FP32, 5184 steps) through the oracle (~1.5 min)."""
    from oracle import fit_oracle as O
    z = load_golden("test001")
    b = z["bounds"]
    g = O.uniform_grid(*b, 50, 50, 150)
    tol = 1e-3 * min(g.dx.min(), g.dy.min(), g.dz.min())
    m = C.test001_boxes_corner_rule(g.x, g.y, g.z, tol)
    s = O.OracleSolver(g, ["pec"] * 3, ["pec"] * 3, solids=[(m, [1.0, 1.0])], bg="pec", dtype=np.float32)
    w = O.OracleWake(wakelength=1.0, q=1e-9, sigmaz=18.5e-3, beta=1.0, skip_cells=12)
    O.wakesolve(s, w, 1.0)
    assert s.Nt == int(z["Nt"])
    assert np.allclose(w.WP[::50], z["WP_samples"], rtol=5e-5, atol=5e-5)
    for f in (np.abs, np.real, np.imag):
        assert np.allclose(f(w.Z)[::20], f(z["Z_samples"]), rtol=5e-4, atol=5e-4)
    assert rel_l2(w.WP, z["WP"]) < 1e-4
