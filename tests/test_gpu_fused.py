"""Fused single-pass step kernel (SolverFIT3D.kernels = 'fused'): the device loop with
ping-pong field buffers must give the two-pass results bit for bit, including the row
crossings of periodic faces, partial tiles, several z ranges per tile column and odd
step counts, and must pass the reference fixtures with the parity tolerances.

The per-cell code is the two-pass code, and the stencil arithmetic is written with
explicitly rounded multiplies, adds and fused multiply-adds, so no kernel variant
depends on the compiler's own contraction choices: fused and two-pass, coded and dense
coefficients all compute the same bits."""

import numpy as np
import pytest
import torch

import cases as C
from oracle_runner import load_golden, rel_l2
from product_runner import run_case

pytestmark = pytest.mark.gpu

FUSED_CASES = ["cavity_f64", "lossy_f64", "lossy_f32", "longitudinal_f64", "skip_nonuniform_f64",
               "periodic_cond_f32"]


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")


def _run(name, kernels, tmp_path, monkeypatch):
    monkeypatch.setenv("WAKIS_GB300_KERNELS", kernels)
    return run_case(name, tmpdir=tmp_path)


@pytest.mark.parametrize("name", FUSED_CASES)
def test_fused_equals_two_pass(name, tmp_path, monkeypatch):
    fused = _run(name, "fused", tmp_path, monkeypatch)
    direct = _run(name, "direct", tmp_path, monkeypatch)
    f64 = C.CASES[name]["dtype"] == "float64"
    for k, v in direct.items():
        if k in ("s", "f", "dt", "Nt"):
            np.testing.assert_array_equal(np.asarray(fused[k]), np.asarray(v), err_msg=f"{name}:{k}")
        else:
            assert close(fused[k], v, f64), (name, k, rel_l2(fused[k], v))
    g = load_golden(name)
    tol = 1e-10 if f64 else 1e-4
    for k in ("WP", "Z"):
        if k in g:
            assert rel_l2(fused[k], g[k]) < tol, (k, rel_l2(fused[k], g[k]))


@pytest.mark.parametrize("bcs,steps", [
    ((["pmc", "periodic", "pec"], ["pec", "periodic", "pml"]), 7),
    ((["periodic", "periodic", "periodic"], ["periodic", "periodic", "periodic"]), 130),
    ((["pec", "pmc", "pec"], ["pml", "pec", "pmc"]), 66),
])
def test_fused_random_fields_all_face_kinds(bcs, steps):
    """Random E, H on a 16 x 12 x 40 grid (a partial tile in x and y; five z ranges per
    tile column), lossy blocks, faces of every kind the fused step serves: the fused
    device loop equals the two-pass device loop to rounding."""
    import wakis_gb300 as wg
    x = np.linspace(-1, 1, 17)
    y = np.linspace(-0.8, 0.7, 13)
    z = np.linspace(-2, 2, 41)
    out = {}
    for kernels in ("direct", "fused"):
        blk = lambda X, Y, Z: (np.abs(X) < 0.4) & (Z > 0.3) & (Z < 1.1)
        grid = wg.GridFIT3D(x=x, y=y, z=z, stl_solids={"blk": blk}, stl_materials={"blk": [2.0, 1.0, 50.0]},
                            verbose=0)
        s = wg.SolverFIT3D(grid, cfln=0.5, bc_low=bcs[0], bc_high=bcs[1], use_stl=True, bg=[1.0, 1.0],
                           dtype=np.float32, n_pml=4, verbose=0)
        s.kernels = kernels
        rng = np.random.default_rng(5)
        s.E.fromarray(rng.standard_normal((s.Nx, s.Ny, s.Nz, 3)).astype(np.float32))
        s.H.fromarray(rng.standard_normal((s.Nx, s.Ny, s.Nz, 3)).astype(np.float32))
        s.emsolve(steps)
        out[kernels] = (s.E.numpy(), s.H.numpy(), s.J.numpy())
    for a, b, k in zip(out["fused"], out["direct"], "EHJ"):
        assert close(a, b, False), (k, rel_l2(a, b))


def close(a, b, f64):
    """Bit-identical (f64 kept for the callers' signature)."""
    return np.array_equal(np.asarray(a), np.asarray(b))


@pytest.mark.parametrize("kernels", ["fused", "direct"])
@pytest.mark.parametrize("name", FUSED_CASES)
def test_coded_coefficients_equal_dense(name, kernels, tmp_path, monkeypatch):
    """The fused step and the two-pass kernels with coded coefficients (a 16-bit code per
    cell into a table of the exact (ch, ce, cl) triples) give the dense kernels' results
    bit for bit."""
    monkeypatch.setenv("WAKIS_GB300_KERNELS", kernels)
    monkeypatch.setenv("WAKIS_GB300_CODES", "1")
    coded = run_case(name, tmpdir=tmp_path)
    monkeypatch.setenv("WAKIS_GB300_CODES", "0")
    dense = run_case(name, tmpdir=tmp_path)
    for k, v in dense.items():
        np.testing.assert_array_equal(np.asarray(coded[k]), np.asarray(v), err_msg=f"{name}:{k}")


def _random_field_solver(x, y, z, dtype, codes, bcs=(["pec", "pmc", "pec"], ["pml", "pec", "pmc"]), bg=(1.0, 1.0)):
    import wakis_gb300 as wg
    blk = lambda X, Y, Z: (np.abs(X) < 0.4) & (Z > 0.3) & (Z < 1.1)
    grid = wg.GridFIT3D(x=x, y=y, z=z, stl_solids={"blk": blk}, stl_materials={"blk": [2.0, 1.0, 50.0]}, verbose=0)
    s = wg.SolverFIT3D(grid, cfln=0.5, bc_low=bcs[0], bc_high=bcs[1], use_stl=True, bg=list(bg), dtype=dtype,
                       n_pml=4, verbose=0)
    s.kernels = "fused"
    s.coefficient_codes = codes
    rng = np.random.default_rng(9)
    s.E.fromarray(rng.standard_normal((s.Nx, s.Ny, s.Nz, 3)).astype(dtype))
    s.H.fromarray(rng.standard_normal((s.Nx, s.Ny, s.Nz, 3)).astype(dtype))
    return s


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_coded_step_random_fields(dtype):
    """Random fields on a 16 x 12 x 40 grid with lossy blocks, PML and PMC faces: coded and
    dense fused device loops agree bit for bit, and the grid is coded."""
    x = np.linspace(-1, 1, 17)
    y = np.linspace(-0.8, 0.7, 13)
    z = np.linspace(-2, 2, 41)
    out = {}
    for codes in (True, False):
        s = _random_field_solver(x, y, z, dtype, codes)
        s.emsolve(33)
        out[codes] = (s.E.numpy(), s.H.numpy(), s.J.numpy(), s.coefficient_code_count)
    assert out[True][3] > 0 and out[False][3] == 0
    for a, b, k in zip(out[True][:3], out[False][:3], "EHJ"):
        np.testing.assert_array_equal(a, b, err_msg=k)


def test_grid_with_too_many_coefficient_triples_stays_dense():
    """48^3 cells with random spacing along every axis have more than 65535 distinct
    coefficient triples: the context stays dense (code count 0) and still steps."""
    rng = np.random.default_rng(4)
    ax = lambda n: np.concatenate([[0.0], np.cumsum(0.5 + rng.random(n))])
    s = _random_field_solver(ax(48) - 24, ax(48) - 24, ax(48) - 24, np.float32, True)
    s.emsolve(4)
    assert s.coefficient_code_count == 0
    assert np.isfinite(s.E.numpy()).all()


# ---------------------------------------------------------------- TMA-fed fused step
@pytest.mark.parametrize("dtype,nx", [(np.float32, 136), (np.float64, 72), (np.float32, 8)])
@pytest.mark.parametrize("staging,rows,ctas", [(1, 4, 3), (2, 4, 3), (1, 8, 2)])
@pytest.mark.parametrize("bcs", [(["pmc", "periodic", "pec"], ["pec", "periodic", "pml"]),
                                 (["periodic", "periodic", "periodic"], ["periodic", "periodic", "periodic"]),
                                 (["pec", "pmc", "pec"], ["pml", "pec", "pmc"])])
def test_tma_staging_equals_loads(dtype, nx, staging, rows, ctas, bcs):
    """The fused step fed by TMA plane rings gives the load-fed fused step's and the
    two-pass kernels' fields bit for bit: random E, H, lossy blocks, an x extent with a
    partial second tile (or a single 8-cell tile), a partial y tile (13 rows), five z
    ranges of 8 planes, every face kind including the periodic row crossings the boxes
    do not hold, and an odd step count."""
    x = np.linspace(-1, 1, nx + 1)
    y = np.linspace(-0.8, 0.7, 14)
    z = np.linspace(-2, 2, 41)
    vec = 4 if dtype == np.float32 else 2
    out = {}
    for mode in ("direct", 0, staging):
        s = _random_field_solver(x, y, z, dtype, True, bcs=bcs)
        if mode == "direct":
            s.kernels = "direct"
        else:
            s.fused_staging = mode
            s._ctx.call("fit_set_fused_shape", vec, rows, 5, ctas)
        s.emsolve(41)
        out[mode] = (s.E.numpy(), s.H.numpy(), s.J.numpy())
        assert s.coefficient_code_count > 0
    for mode in (0, staging):
        for a, b, k in zip(out[mode], out["direct"], "EHJ"):
            np.testing.assert_array_equal(a, b, err_msg=f"staging {mode}: {k}")


@pytest.mark.parametrize("name", ["cavity_f64", "lossy_f32", "periodic_cond_f32", "longitudinal_f64"])
def test_tma_staging_reference_cases(name, tmp_path, monkeypatch):
    """Wake runs of the reference fixtures with the TMA-fed fused step: bit-identical to
    the two-pass kernels, so within the parity tolerances of the fixtures."""
    monkeypatch.setenv("WAKIS_GB300_STAGING", "1")
    tma = _run(name, "fused", tmp_path, monkeypatch)
    monkeypatch.setenv("WAKIS_GB300_STAGING", "0")
    direct = _run(name, "direct", tmp_path, monkeypatch)
    for k, v in direct.items():
        np.testing.assert_array_equal(np.asarray(tma[k]), np.asarray(v), err_msg=f"{name}:{k}")


def test_tma_staging_rejected_where_it_does_not_apply():
    """Nx not a multiple of 8, or dense coefficients: fit_set_fused_staging refuses and the
    solver keeps the load-fed step."""
    import wakis_gb300 as wg
    from wakis_gb300 import _native as nat
    s = _random_field_solver(np.linspace(-1, 1, 13), np.linspace(-0.8, 0.7, 14), np.linspace(-2, 2, 41),
                             np.float32, True)
    s._sync_coeffs()
    s._ensure_codes()
    with pytest.raises(nat.FitError):
        s._ctx.call("fit_set_fused_staging", 1, 1)
    s2 = _random_field_solver(np.linspace(-1, 1, 17), np.linspace(-0.8, 0.7, 14), np.linspace(-2, 2, 41),
                              np.float32, False)
    s2._sync_coeffs()
    s2._ensure_codes()
    with pytest.raises(nat.FitError):
        s2._ctx.call("fit_set_fused_staging", 1, 1)
    assert isinstance(s2, wg.SolverFIT3D)


# ---------------------------------------------------------------- cell pairs
_GROUP_BCS = [(["pmc", "periodic", "pec"], ["pec", "periodic", "pml"]),
              (["periodic", "periodic", "periodic"], ["periodic", "periodic", "periodic"]),
              (["pec", "pmc", "pec"], ["pml", "pec", "pmc"])]


@pytest.mark.parametrize("dtype,nx,ny,nz,bcs", [
    (np.float32, 17, 13, 40, 0), (np.float32, 17, 13, 40, 1), (np.float32, 17, 13, 40, 2),
    (np.float64, 17, 13, 40, 0), (np.float64, 17, 13, 40, 1), (np.float64, 17, 13, 40, 2),
    (np.float32, 15, 7, 20, 2), (np.float32, 1, 5, 8, 1), (np.float64, 3, 3, 6, 1)])
def test_cell_groups_equal_row_vectors(dtype, nx, ny, nz, bcs):
    """The coded two-pass passes on flat-index cell pairs (Nx odd, N even) against the
    dense two-pass passes on single cells: random E, H, lossy blocks, every face kind
    including the periodic row and plane crossings a pair straddles (Nx = 1: every pair
    spans two rows), an odd step count; bit for bit."""
    x = np.linspace(-1, 1, nx + 1)
    y = np.linspace(-0.8, 0.7, ny + 1)
    z = np.linspace(-2, 2, nz + 1)
    out = {}
    for codes in (True, False):
        # a lossy background (tau = eps/sigma above dt) keeps every cell conductive, so tiny
        # grids that the block misses still run the loss-factor step
        s = _random_field_solver(x, y, z, dtype, codes, bcs=_GROUP_BCS[bcs], bg=(1.5, 1.0, 1e-3))
        s.kernels = "direct"
        s.emsolve(21)
        out[codes] = (s.E.numpy(), s.H.numpy(), s.J.numpy(), s.coefficient_code_count)
    assert out[True][3] > 0 and out[False][3] == 0
    for a, b, k in zip(out[True][:3], out[False][:3], "EHJ"):
        np.testing.assert_array_equal(a, b, err_msg=k)
