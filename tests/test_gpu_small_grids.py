"""Degenerate and ragged grids: 1-, 2- and 3-cell axes, odd sizes (every vector width
and partial tiles of the fused step), random fields, conductive backgrounds and every
face kind that needs no PML depth, stepped by emsolve (the device loop) and checked
against the CPU oracle step for step."""

import numpy as np
import pytest
import torch

from oracle import fit_oracle as O
from oracle_runner import rel_l2

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1, 3), (2, 1, 4), (1, 3, 2), (3, 2, 5), (5, 4, 3), (2, 2, 2), (4, 3, 7), (7, 6, 9)]
FACES = [(["pec"] * 3, ["pec"] * 3),
         (["periodic", "pec", "pmc"], ["periodic", "pec", "pec"]),
         (["pmc", "periodic", "pec"], ["pec", "periodic", "abc"]),
         (["abc", "pmc", "periodic"], ["pec", "pec", "periodic"])]


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("faces", range(len(FACES)))
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_small_grid_against_oracle(shape, faces, dtype):
    import wakis_gb300 as wg
    nx, ny, nz = shape
    lo, hi = FACES[faces]
    rng = np.random.default_rng(hash((shape, faces)) % (2 ** 32))
    x = np.cumsum(np.r_[0.0, rng.uniform(0.5, 1.5, nx)])
    y = np.cumsum(np.r_[0.0, rng.uniform(0.5, 1.5, ny)])
    z = np.cumsum(np.r_[0.0, rng.uniform(0.5, 1.5, nz)])
    bg = [1.5, 1.0, 1e-3]  # tau = eps/sigma stays above dt: a well-conditioned loss factor
    steps = 9
    s = wg.SolverFIT3D(wg.GridFIT3D(x=x, y=y, z=z, verbose=0), cfln=0.5, bc_low=lo, bc_high=hi, use_stl=False,
                       bg=bg, dtype=dtype, verbose=0)
    o = O.OracleSolver(O.OracleGrid(x, y, z), lo, hi, bg=bg, cfln=0.5, dtype=dtype)
    assert float(s.dt) == float(o.dt)
    n = nx * ny * nz
    E0 = rng.standard_normal(3 * n).astype(dtype)
    H0 = rng.standard_normal(3 * n).astype(dtype)
    s.E.fromarray(E0)
    s.H.fromarray(H0)
    o.E[:] = E0
    o.H[:] = H0
    n_axes = (nx, ny, nz)
    if any(lo[a] == "abc" and n_axes[a] < 2 for a in range(3)):
        with pytest.raises(IndexError):  # the reference's ABC update indexes plane 1
            O.emsolve(o, steps)
        with pytest.raises(IndexError):
            s.emsolve(steps)
        return
    s.emsolve(steps)
    O.emsolve(o, steps)
    tol = 1e-10 if dtype == np.float64 else 2e-5
    for k, a, b in (("E", s.E.numpy(), o.E), ("H", s.H.numpy(), o.H), ("J", s.J.numpy(), o.J)):
        if np.any(b):
            assert rel_l2(a, b) < tol, (shape, faces, k, rel_l2(a, b))
        else:
            assert not np.any(a), (shape, faces, k)
