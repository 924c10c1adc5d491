"""Ez line history export (wakesolve(save_Ez=True)): the device-recorded slabs
E_z(xx, yy, :) before every step equal the oracle's recorded slabs (the reference's
Ez.h5 datasets) within the parity tolerance, with the reference's keys, and read_Ez
reads the file back."""

import numpy as np
import pytest
import torch

import cases as C
from oracle import fit_oracle as O
from oracle_runner import oracle_solver, rel_l2
from product_runner import make_grid, make_solver

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")


@pytest.mark.parametrize("name", ["cavity_f64", "lossy_f32", "longitudinal_f64"])
def test_ez_history_matches_oracle(name, tmp_path):
    import wakis_gb300 as wg
    case = C.CASES[name]
    grid = make_grid(wg, case)
    wake = wg.WakeSolver(wakelength=case["wakelength"], save=False, verbose=0, results_folder=str(tmp_path),
                         Ez_file=str(tmp_path / "Ez.h5"), **case["wake"])
    s = make_solver(wg, case, grid, wake)
    s.wakesolve(wakelength=case["wakelength"], compute_plane=case["compute_plane"], save_Ez=True)
    wp = wake.WP.copy()
    w2 = wg.WakeSolver(wakelength=case["wakelength"], save=False, verbose=0, results_folder=str(tmp_path),
                       **case["wake"])
    hf = w2.read_Ez(wake.Ez_file, return_value=True)
    assert {"x", "y", "z", "dx", "dy", "dz", "t"} <= set(hf.keys())
    np.testing.assert_array_equal(w2.t, wake.t)
    np.testing.assert_array_equal(w2.zf, s.z)

    os_ = oracle_solver(case)
    ow = O.OracleWake(wakelength=case["wakelength"], **case["wake"])
    slabs = O.wakesolve(os_, ow, case["wakelength"], case["compute_plane"])
    assert len([k for k in hf.keys() if k.startswith("#")]) == len(slabs) == s.Nt
    got = np.stack([np.asarray(hf["#" + str(n).zfill(5)], dtype=np.float64) for n in range(s.Nt)])
    assert got.shape == slabs.shape
    tol = 1e-10 if case["dtype"] == "float64" else 1e-3
    assert rel_l2(got, slabs) < tol
    assert rel_l2(wp, ow.WP) < (1e-10 if case["dtype"] == "float64" else 1e-4)


@pytest.mark.parametrize("name", ["cavity_f64", "lossy_f32", "longitudinal_f64"])
def test_save_J_matches_oracle(name, tmp_path, monkeypatch):
    """wakesolve(save_J=True) writes Jz (the reference's Jz.h5 datasets) in the working
    directory: J_z on the wake lines after the beam update and before each step (the beam
    current on the beam line, sigma*E of the previous step on a conductive grid).  The
    run itself gives the same wake as the device loop."""
    import wakis_gb300 as wg
    monkeypatch.chdir(tmp_path)
    case = C.CASES[name]
    wake = wg.WakeSolver(wakelength=case["wakelength"], save=False, verbose=0, results_folder=str(tmp_path),
                         **case["wake"])
    s = make_solver(wg, case, make_grid(wg, case), wake)
    s.wakesolve(wakelength=case["wakelength"], compute_plane=case["compute_plane"], save_J=True)
    w2 = wg.WakeSolver(wakelength=case["wakelength"], save=False, verbose=0, **case["wake"])
    fname = "Jz.h5" if (tmp_path / "Jz.h5").exists() else "Jz.npz"
    hf = w2.read_Ez(str(tmp_path / fname), return_value=True)
    assert {"x", "y", "z", "dx", "dy", "dz", "t"} <= set(hf.keys())
    got = np.stack([np.asarray(hf["#" + str(n).zfill(5)], dtype=np.float64) for n in range(s.Nt)])

    os_ = oracle_solver(case)
    ow = O.OracleWake(wakelength=case["wakelength"], **case["wake"])
    jref = []
    O.wakesolve(os_, ow, case["wakelength"], case["compute_plane"], j_slabs=jref)
    jref = np.array(jref)
    assert got.shape == jref.shape
    assert np.abs(jref).max() > 0
    tol = 1e-10 if case["dtype"] == "float64" else 1e-3
    assert rel_l2(got, jref) < tol
    assert rel_l2(wake.WP, ow.WP) < (1e-10 if case["dtype"] == "float64" else 1e-4)
