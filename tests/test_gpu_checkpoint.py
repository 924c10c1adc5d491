"""Checkpoints and the emsolve save path against the reference's own behaviour
(fixtures tests/golden/checkpoint_*.npz and emsolve_save.npz, written by running the
reference in tests/golden/make_golden.py):

* save_state after 17 steps of a beam user loop on a lossy PMC/PEC grid: the saved
  datasets (keys H, E, J, FP64, 3N values each) equal the reference's within the FP64
  parity tolerance; a fresh solver that loads them and runs the remaining steps ends
  where the reference's restarted and uninterrupted runs end, and where this solver's
  own uninterrupted run ends; reset_fields zeroes E, H and J;
* restarts whose stored J is zero or sigma*E continue on the folded-J step and equal the
  uninterrupted run bit for bit;
* emsolve(save=True) raises the reference's TypeError, before any step.
"""

import os

import numpy as np
import pytest
import torch

import cases as C
from oracle_runner import load_golden, rel_l2
from product_runner import make_grid, make_solver

pytestmark = pytest.mark.gpu
TOL64 = 1e-10


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")


def _beam_steps(wg, s, beam, n0, n1):
    for n in range(n0, n1):
        beam.update(s, n * s.dt)
        s.one_step()


@pytest.mark.parametrize("name", list(C.CHECKPOINT_CASES))
def test_checkpoint_restart_matches_reference(name, tmp_path):
    import wakis_gb300 as wg
    spec = C.CHECKPOINT_CASES[name]
    case = C.CASES[spec["base"]]
    ref = load_golden(name)
    n1, nt = spec["save_at"], case["Nt"]
    s1 = make_solver(wg, case, make_grid(wg, case))
    b1 = wg.sources.Beam(**case["beam"])
    _beam_steps(wg, s1, b1, 0, n1)
    fname = str(tmp_path / "state.h5")
    s1.save_state(fname)
    st = s1.read_state(fname)
    assert sorted(st.keys()) == list(ref["keys"])
    for k in ref["keys"]:
        a = np.asarray(st[k])
        assert a.dtype == ref["saved_" + k].dtype and a.shape == ref["saved_" + k].shape, k
        assert rel_l2(a, ref["saved_" + k]) < TOL64, (k, rel_l2(a, ref["saved_" + k]))
    st.close()
    s2 = make_solver(wg, case, make_grid(wg, case))
    s2.load_state(fname)
    _beam_steps(wg, s2, wg.sources.Beam(**case["beam"]), n1, nt)
    _beam_steps(wg, s1, b1, n1, nt)
    for k in ("E", "H", "J"):
        got = getattr(s2, k).numpy()
        assert rel_l2(got, ref["restart_" + k]) < TOL64, (k, rel_l2(got, ref["restart_" + k]))
        assert rel_l2(got, ref["cont_" + k]) < TOL64
        # the first step after a load reads the stored J (the beam line holds the beam
        # current, not sigma*E) where the uninterrupted run folds J = sigma*E into the loss
        # factor: the two differ by rounding only
        assert rel_l2(got, getattr(s1, k).numpy()) < 1e-13
    s2.reset_fields()
    assert float(ref["reset_max"]) == 0.0
    for k in ("E", "H", "J"):
        assert not np.any(getattr(s2, k).numpy())


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("bg", [[1.0, 1.0], [2.0, 1.0, 0.3]])
def test_restart_is_bit_exact_when_J_is_zero_or_sigma_E(dtype, bg, tmp_path):
    """Random fields on a PEC box, free emsolve runs (device loop): save after 30 steps,
    load into a fresh solver, 50 more steps; lossless (J = 0) and conductive (J = sigma*E)
    grids give the uninterrupted run's E, H and J bit for bit."""
    import wakis_gb300 as wg

    def solver():
        g = wg.GridFIT3D(-1, 1, -1, 1, -1, 1, 12, 10, 16, verbose=0)
        s = wg.SolverFIT3D(g, cfln=0.5, bc_low=["pec"] * 3, bc_high=["pec"] * 3, bg=bg, dtype=dtype, verbose=0)
        return s

    s1 = solver()
    rng = np.random.default_rng(3)
    s1.E.fromarray(rng.standard_normal(3 * s1.N).astype(dtype))
    s1.H.fromarray(rng.standard_normal(3 * s1.N).astype(dtype))
    s1.emsolve(30)
    fname = str(tmp_path / "state.h5")
    s1.save_state(fname)
    s2 = solver()
    s2.load_state(fname)  # its first step zeroes the ghost planes again: they are zero already
    s2.emsolve(50)
    s1.emsolve(50)
    for k in ("E", "H", "J"):
        np.testing.assert_array_equal(getattr(s2, k).numpy(), getattr(s1, k).numpy(), err_msg=k)


def test_emsolve_save_raises_like_reference(tmp_path, monkeypatch):
    import wakis_gb300 as wg
    ref = load_golden("emsolve_save")
    spec = C.EMSOLVE_SAVE_CASE
    g = spec["grid"]
    grid = wg.GridFIT3D(g["xmin"], g["xmax"], g["ymin"], g["ymax"], g["zmin"], g["zmax"], g["Nx"], g["Ny"], g["Nz"],
                        verbose=0)
    s = wg.SolverFIT3D(grid, bc_low=["pec"] * 3, bc_high=["pec"] * 3, verbose=0)
    monkeypatch.chdir(tmp_path)
    with pytest.raises(Exception) as ei:
        s.emsolve(spec["Nt"], save=True, fields=spec["fields"], components=spec["components"])
    assert type(ei.value).__name__ == str(ref["exc_type"])
    assert str(ei.value) == str(ref["exc_msg"])
    assert s.nstep == int(ref["nstep"]) and s.Nt == spec["Nt"]
    try:
        import h5py  # noqa: F401
        assert sorted(os.listdir(tmp_path)) == list(ref["files"])
    except ImportError:
        pass
