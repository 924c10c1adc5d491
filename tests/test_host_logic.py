"""CPU tests of the host side: the C-ABI library loads and exports every declared entry
point, and the host logic (grid metrics, masks, Field indexing, tap tables, step-time
types, boundary codes) matches the oracle.  No GPU compute is called."""

import ctypes
import os
import re

import numpy as np
import pytest
import torch

import cases as C
from oracle import fit_oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "wakis_fit.h")).read()
    return re.findall(r"FIT_API\s+\w+\s+(fit_\w+)\s*\(", txt)


def test_library_builds_and_exports_all_symbols():
    from wakis_gb300 import _native as nat
    lib = nat.load()
    names = declared_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) == set(nat.exported_symbols())
    buf = ctypes.create_string_buffer(128)
    assert lib.fit_version(buf, 128) == 0
    assert b"sm_103a" in buf.value


def test_ctx_create_rejects_bad_arguments_without_gpu():
    from wakis_gb300 import _native as nat
    lib = nat.load()
    d = nat.FitGridDesc()
    d.nx, d.ny, d.nz = 0, 4, 4
    h = ctypes.c_void_p()
    rc = lib.fit_ctx_create(ctypes.byref(d), ctypes.byref(h))
    assert rc == -1 and "dimensions" in nat.last_error(None)
    d.nx = 4
    d.dtype = 7
    assert lib.fit_ctx_create(ctypes.byref(d), ctypes.byref(h)) == -1
    if not torch.cuda.is_available():
        d.dtype = 0
        assert lib.fit_ctx_create(ctypes.byref(d), ctypes.byref(h)) == -6  # no device
    # cells are addressed by 32-bit offsets within a component: N + Nx*Ny < 2^31
    d.dtype = 0
    d.nx, d.ny, d.nz = 1290, 1290, 1290  # N = 2146689000 < 2^31, N + Nx*Ny above it: refused
    assert lib.fit_ctx_create(ctypes.byref(d), ctypes.byref(h)) == -1
    assert "too large" in nat.last_error(None)
    d.nx, d.ny, d.nz = 32768, 32768, 2  # N = 2^31: refused
    assert lib.fit_ctx_create(ctypes.byref(d), ctypes.byref(h)) == -1
    d.nx, d.ny, d.nz = 16384, 16384, 7  # N + Nx*Ny = 2^31 exactly: refused
    assert lib.fit_ctx_create(ctypes.byref(d), ctypes.byref(h)) == -1
    assert "too large" in nat.last_error(None)


def test_bc_codes():
    from wakis_gb300 import _native as nat
    assert nat.bc_code("PEC") == nat.bc_code("electric") == 1
    assert nat.bc_code("pmc") == nat.bc_code("Magnetic") == 3
    with pytest.raises(ValueError):
        nat.bc_code("mpi")


@pytest.mark.parametrize("name", ["mixed_bc_f64", "cavity_f64", "longitudinal_f64"])
def test_grid_metrics_match_oracle(name):
    import wakis_gb300 as wg
    case = C.CASES[name]
    x, y, z = C.axes(case)
    g = wg.GridFIT3D(x=x, y=y, z=z, verbose=0)
    o = O.OracleGrid(x, y, z)
    for attr in ("L", "iA", "tL", "itA"):
        np.testing.assert_array_equal(getattr(g, attr).numpy(), getattr(o, attr), err_msg=attr)


def test_solid_masks_center_and_corner_rules():
    import wakis_gb300 as wg
    case = C.CASES["cavity_f64"]
    x, y, z = C.axes(case)
    X, Y, Z = C.centres(x, y, z)
    ref = C.cube_pipe(X, Y, Z)
    g = wg.GridFIT3D(x=x, y=y, z=z, stl_solids={"c": C.cube_pipe}, stl_materials={"c": "vacuum"},
                     stl_method="center", verbose=0)
    np.testing.assert_array_equal(g.grid["c"], ref.reshape(-1))
    assert g.stl_materials["c"] == [1.0, 1.0]
    # corner rule on the test_001 boxes
    gx = np.linspace(-0.025, 0.025, 11)
    gz = np.linspace(-0.05, 0.05, 21)
    boxes = lambda X, Y, Z: (((np.abs(X) <= 0.025) & (np.abs(Y) <= 0.025) & (np.abs(Z) <= 0.015))
                             | ((np.abs(X) <= 0.0075) & (np.abs(Y) <= 0.0075) & (np.abs(Z) <= 0.05)))
    g2 = wg.GridFIT3D(x=gx, y=gx, z=gz, stl_solids={"c": boxes}, stl_materials={"c": [1.0, 1.0]}, verbose=0)
    np.testing.assert_array_equal(g2.grid["c"].reshape(10, 10, 20), C.test001_boxes_corner_rule(gx, gx, gz, 0.0))
    with pytest.raises(NotImplementedError):
        wg.GridFIT3D(x=gx, y=gx, z=gz, stl_solids={"c": "cavity.stl"}, stl_materials={"c": "vacuum"}, verbose=0)


def test_field_layout_and_indexing_cpu():
    from wakis_gb300 import Field
    rng = np.random.default_rng(0)
    f = Field(4, 3, 5)
    a = rng.standard_normal(3 * 60)
    f.fromarray(a)
    for d, c in enumerate("xyz"):
        m = a[d * 60:(d + 1) * 60].reshape((4, 3, 5), order="F")
        np.testing.assert_array_equal(f[:, :, :, c], m)
        np.testing.assert_array_equal(f[1, :, -1, c], m[1, :, -1])
        np.testing.assert_array_equal(f[::-1, 0, 2, c], m[::-1, 0, 2])
    f[2, 1, 3, "y"] = 7.0
    assert f.array[60 + 2 + 4 * 1 + 12 * 3].item() == 7.0
    b = f.numpy()
    np.testing.assert_allclose(f[:, :, :, "Abs"],
                               np.sqrt(sum(b[d * 60:(d + 1) * 60].reshape((4, 3, 5), order="F") ** 2
                                           for d in range(3))))
    calls = []
    f._on_write = lambda fld: calls.append(fld[2, 1, 3, "y"])
    f[2, 1, 3, "y"] = 9.0
    assert calls == [7.0]  # the hook runs before the storage changes
    with pytest.raises(IndexError):
        f[0, 0, 0]
    assert f.compute_ijk(2 + 4 * 1 + 12 * 3) == (2, 1, 3)


def test_step_times_follow_reference_scalar_types():
    from wakis_gb300.routines import _step_times
    for dt in (np.float32(1.9e-12), np.float64(1.9e-12), 1.9e-12):
        t = _step_times(dt, 5000)
        v = 0.8 * 299792458.0
        vt = v * t
        for n in (0, 1, 77, 4999):
            assert (v * (n * dt)) == vt[n]
            assert type(v * (n * dt)) in (type(vt[n]), float)


@pytest.mark.parametrize("name", ["cavity_f64", "skip_nonuniform_f64", "longitudinal_f64", "lossy_f32", "counter_f64"])
def test_tap_table_reproduces_reference_loop(name):
    """The per-step (m, k0, cnt) table adds exactly the reference's terms: each valid
    (s index, z index) pair once, at the step of its time index, with the reference's dz
    factor (negated and read from the loop index of a counter-moving test charge)."""
    import wakis_gb300 as wg
    case = C.CASES[name]
    x, y, z = C.axes(case)
    g = O.OracleGrid(x, y, z)
    dtype = np.float32 if case["dtype"] == "float32" else np.float64
    s = O.OracleSolver(g, case["bc_low"], case["bc_high"], solids=[(m, mat) for _, m, mat in C.solids_for(case)],
                       bg=case["bg"], cfln=case["cfln"], dtype=dtype, n_pml=case.get("n_pml", 10))
    w = wg.WakeSolver(wakelength=case["wakelength"], save=False, verbose=0, **case["wake"])
    ow = O.OracleWake(wakelength=case["wakelength"], **case["wake"])
    tmax = (case["wakelength"] + w.ti * w.v + (s.z.max() - s.z.min())) / w.v
    Nt = int(tmax / s.dt)
    w.t = np.arange(0, Nt * s.dt, s.dt)
    w.zf, w.dz = s.z, g.dz
    ow.t, ow.zf, ow.dz = w.t, s.z, g.dz
    longitudinal = case["compute_plane"] == "longitudinal"
    sv, it, valid, kskip, nz, nt, wdz = w._tap_index(Nt, longitudinal, g.Nz)
    counter = bool(case["wake"].get("counter_moving")) and not longitudinal
    so, ito, valido, _, _ = O.wp_index_table(ow, Nt, counter)
    dzo = np.asarray(g.dz, dtype=np.float64)[:nz]
    if counter:  # the oracle's table is in loop order: loop index k reads z index nz-1-k
        ito, valido, dzo = ito[:, ::-1], valido[:, ::-1], (-1 * dzo)[::-1]
    np.testing.assert_array_equal(wdz, dzo)
    np.testing.assert_array_equal(sv, so)
    np.testing.assert_array_equal(valid, valido)
    np.testing.assert_array_equal(np.where(valid, it, 0), np.where(valido, ito, 0))
    row_ptr, em, ek0, ecnt = w._tap_csr(it, valid, Nt)
    # replay: term order per m must be k ascending, each valid (m, k) exactly once
    seen = {}
    for n in range(Nt):
        for e in range(row_ptr[n], row_ptr[n + 1]):
            for c in range(ecnt[e]):
                k = ek0[e] + c
                assert it[em[e], k] == n
                seen.setdefault(int(em[e]), []).append(int(k))
    for m in range(len(sv)):
        ks = list(np.nonzero(valid[m])[0])
        if counter:  # the reference's loop reads z downwards; so do the steps
            ks = ks[::-1]
        assert seen.get(m, []) == ks


def test_solver_without_a_device_raises_import_error():
    """The reference raises ImportError when its GPU stack is missing
    (wakis/solverFIT3D.py:365); a solver without a CUDA device does the same."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    import wakis_gb300 as wg
    grid = wg.GridFIT3D(0, 1, 0, 1, 0, 1, 4, 4, 4, verbose=0)
    with pytest.raises(ImportError):
        wg.SolverFIT3D(grid, verbose=0)
