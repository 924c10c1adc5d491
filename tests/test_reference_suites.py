"""Ports of the reference's own test suites for this path, run against wakis_gb300:

* tests/test_004_wakes_and_impedances.py (CPU): the WakeSolver FFT utilities turn a
  sinusoidal wake into an impedance peak of the right height and frequency and back;
* tests/test_005_pml_boundaries.py (GPU): a plane wave into a 30-cell PML on a
  20 x 20 x 200 FP32 grid (vacuum, eps_r=3 with sigma=1, sigma=1) reflects less than
  10 % -- the same user loop (planeWave.update + one_step), sizes and bounds.
"""

import numpy as np
import pytest
from scipy.constants import c, mu_0


def _sin_wake():
    fr, A = 0.5e9, 100
    t = np.linspace(0, 100 * 1e-9, 3000)
    return fr, A, t, A * np.sin(2 * np.pi * fr * t)


def test_004_sin_wake_round_trip():
    from wakis_gb300 import WakeSolver as wk
    fr, A, t, wake = _sin_wake()
    f, Z = wk.calc_impedance_from_wake([t, wake])
    tt, wwake = wk.calc_wake_from_impedance([f, Z], samples=3000)
    ff, Zz = wk.calc_impedance_from_wake([tt, wwake])
    ttt, wwwake = wk.calc_wake_from_impedance([ff, Zz], samples=3000)
    assert np.allclose(wake, wwake, atol=1)
    assert np.allclose(wake, wwwake, atol=1)


def test_004_sin_impedance_peak():
    from wakis_gb300 import WakeSolver as wk
    fr, A, t, wake = _sin_wake()
    f, Z = wk.calc_impedance_from_wake([t, wake])
    tt, wwake = wk.calc_wake_from_impedance([f, Z], samples=3000)
    ff, Zz = wk.calc_impedance_from_wake([tt, wwake])
    assert np.allclose(np.max(np.abs(Z)), A, atol=1)
    assert np.allclose(np.max(np.abs(Zz)), A, atol=1)
    assert np.allclose(f[np.argmax(Z)], fr, atol=1e6)
    assert np.allclose(ff[np.argmax(Zz)], fr, atol=1e6)


@pytest.mark.gpu
@pytest.mark.parametrize("eps_r,sigma", [(1.0, 0.0), (3.0, 1.0), (1.0, 1.0)])
def test_005_pml_reflection_planewave(eps_r, sigma):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    import wakis_gb300 as wakis
    xmin, xmax, ymin, ymax, zmin, zmax = -1.0, 1.0, -1.0, 1.0, 0.0, 1.0
    Nx, Ny, Nz = 20, 20, 200
    grid = wakis.GridFIT3D(xmin, xmax, ymin, ymax, zmin, zmax, Nx, Ny, Nz, verbose=0)
    solver = wakis.SolverFIT3D(grid, use_stl=False, bg=[eps_r, 1.0, sigma], bc_low=["periodic", "periodic", "pec"],
                               bc_high=["periodic", "periodic", "pml"], n_pml=30, dtype=np.float32, verbose=0)
    amplitude, nodes = 100.0, 7
    f = 15 / ((solver.z.max() - solver.z.min()) / c)
    plane = wakis.sources.PlaneWave(xs=slice(0, Nx), ys=slice(0, Ny), zs=0, beta=1.0, amplitude=amplitude, f=f,
                                    nodes=nodes, phase=np.pi / 2)
    solver.dt = 1 / f / 200
    z_pml = 0
    for k in range(solver.n_pml):
        z_pml += solver.dz[Nz - 1 - k]
    Nt = int(eps_r * 2.0 * (zmax - zmin - z_pml) / c / solver.dt)
    for n in range(Nt):
        plane.update(solver, n * solver.dt)
        solver.one_step()
    reflection_h = solver.H.get_abs()[Nx // 2, Ny // 2, :].max()
    reflection_e = solver.E.get_abs()[Nx // 2, Ny // 2, :].max() / (mu_0 * c)
    assert reflection_h <= 10, f"PML H reflection >10% with eps_r={eps_r}, sigma={sigma}"
    assert reflection_e <= 10, f"PML E reflection >10% with eps_r={eps_r}, sigma={sigma}"
