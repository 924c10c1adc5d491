"""WakeSolver post-processing of an Ez file without a live run (calc_long_WP,
calc_long_WP_3d, solve): the wake integral runs on the device in the reference's
operation order, so s and WP / WP_3d equal the oracle's (the reference's scalar loops)
bit for bit; WPx / WPy and the impedances agree within FP64 rounding.  Inputs are seeded
synthetic Ez line histories written with the reference's Ez.h5 keys (as .npz), plus a
live run's own export.  The error cases mirror the reference's exceptions and need no GPU."""

import numpy as np
import pytest
import torch
from scipy.constants import c as c_light

import cases as C
from oracle import fit_oracle as O
from oracle_runner import load_golden, rel_l2

gpu = pytest.mark.gpu


def synthetic_history(seed, nz=40, nt=320, shape3=True, t0=0.0, beta=1.0):
    """A recorded Ez history with a non-uniform dz and the reference's file keys."""
    rng = np.random.default_rng(seed)
    dz = 1e-3 * (0.8 + 0.4 * rng.random(nz))
    zedges = np.concatenate([[-0.02], -0.02 + np.cumsum(dz)])
    z = 0.5 * (zedges[1:] + zedges[:-1])
    dt = 0.45 * dz.min() / c_light
    t = t0 + np.arange(0, nt * dt, dt)[:nt]
    x = np.array([-1.1e-3, 0.0, 0.9e-3])
    y = np.array([-0.8e-3, 0.0, 1.2e-3])
    shape = (nt, 3, 3, nz) if shape3 else (nt, nz)
    slabs = rng.standard_normal(shape).astype(np.float32).astype(np.float64) * 1e3
    return dict(x=x, y=y, z=z, dx=np.full(3, 1e-3), dy=np.full(3, 1e-3), dz=dz, t=t), slabs


def write_file(path, meta, slabs):
    data = dict(meta)
    for n in range(len(slabs)):
        data["#" + str(n).zfill(5)] = slabs[n]
    np.savez(path, **data)
    return str(path)


def oracle_wake(meta, slabs, plane, **kw):
    ow = O.OracleWake(**kw)
    ow.t, ow.zf, ow.dz, ow.xf, ow.yf = meta["t"], meta["z"], meta["dz"], meta["x"], meta["y"]
    O.postprocess(ow, slabs, plane)
    return ow


WAKE = dict(q=1e-9, sigmaz=2e-3, wakelength=0.02)


def need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")


@gpu
@pytest.mark.parametrize("skip,beta,t0,nt", [(0, 1.0, 0.0, 320), (3, 1.0, 0.0, 320), (0, 0.8, 0.0, 320),
                                             (2, 1.0, 12e-12, 320), (1, 1.0, 0.0, 200)])
def test_solve_from_file_3d_matches_oracle(tmp_path, skip, beta, t0, nt):
    """t0 > 0 makes the first taps' time index negative (the reference's Python index then
    wraps to the end of the history); nt = 200 leaves the late taps outside the history."""
    need_gpu()
    import wakis_gb300 as wg
    meta, slabs = synthetic_history(11 + skip, t0=t0, beta=beta, nt=nt)
    fname = write_file(tmp_path / "Ez.npz", meta, slabs)
    w = wg.WakeSolver(save=False, verbose=0, Ez_file=fname, skip_cells=skip, beta=beta, **WAKE)
    w.solve()
    ow = oracle_wake(meta, slabs, "both", skip_cells=skip, beta=beta, **WAKE)
    np.testing.assert_array_equal(w.s, ow.s)
    np.testing.assert_array_equal(w.WP_3d, ow.WP_3d)
    np.testing.assert_array_equal(w.WP, ow.WP)
    assert rel_l2(w.WPx, ow.WPx) < 1e-12 and rel_l2(w.WPy, ow.WPy) < 1e-12
    np.testing.assert_array_equal(w.f, ow.f)
    for k in ("Z", "Zx", "Zy"):
        assert rel_l2(getattr(w, k), getattr(ow, k)) < 1e-10, k
    assert w.Ez_hf is None  # closed as the reference closes it


@gpu
def test_calc_long_WP_from_1d_file_matches_oracle(tmp_path):
    need_gpu()
    import wakis_gb300 as wg
    meta, slabs = synthetic_history(5, shape3=False)
    fname = write_file(tmp_path / "Ez.npz", meta, slabs)
    w = wg.WakeSolver(save=False, verbose=0, Ez_file=fname, **WAKE)
    w.solve(compute_plane="longitudinal")
    ow = oracle_wake(meta, slabs, "longitudinal", **WAKE)
    np.testing.assert_array_equal(w.s, ow.s)
    np.testing.assert_array_equal(w.WP, ow.WP)
    assert rel_l2(w.Z, ow.Z) < 1e-10
    np.testing.assert_array_equal(w.Ezt, slabs.T)


@gpu
@pytest.mark.parametrize("skip", [0, 4])
def test_calc_long_WP_on_3d_slabs_takes_the_corner_line(tmp_path, skip):
    """calc_long_WP on 3x3 slabs integrates Ez[sh0//2 + 1, sh1//2 + 1, zz] (the reference's
    index), not the centre line."""
    need_gpu()
    import wakis_gb300 as wg
    meta, slabs = synthetic_history(7)
    fname = write_file(tmp_path / "Ez.npz", meta, slabs)
    w = wg.WakeSolver(save=False, verbose=0, Ez_file=fname, skip_cells=skip, **WAKE)
    w.calc_long_WP()
    zz = slice(skip, -skip) if skip else slice(None)
    ow = oracle_wake(meta, slabs[:, 2, 2, zz], "longitudinal", skip_cells=skip, **WAKE)
    np.testing.assert_array_equal(w.WP, ow.WP)


@gpu
@pytest.mark.parametrize("name", ["cavity_f64", "lossy_f32"])
def test_live_run_export_post_processed_again(name, tmp_path):
    """wakesolve(save_Ez=True), then a fresh WakeSolver solves from the exported file: the
    same s, and WP within the difference of the live run's compensated sums and the
    reference's plain sums."""
    need_gpu()
    import cases as C
    import wakis_gb300 as wg
    from product_runner import make_grid, make_solver
    case = C.CASES[name]
    wake = wg.WakeSolver(wakelength=case["wakelength"], save=False, verbose=0, results_folder=str(tmp_path),
                         Ez_file=str(tmp_path / "Ez.h5"), **case["wake"])
    s = make_solver(wg, case, make_grid(wg, case), wake)
    s.wakesolve(wakelength=case["wakelength"], compute_plane=case["compute_plane"], save_Ez=True)
    w2 = wg.WakeSolver(wakelength=case["wakelength"], save=False, verbose=0, Ez_file=wake.Ez_file,
                       **case["wake"])
    w2.solve(compute_plane=case["compute_plane"])
    np.testing.assert_array_equal(w2.s, wake.s)
    assert rel_l2(w2.WP, wake.WP) < 1e-12
    assert rel_l2(w2.WP_3d, wake.WP_3d) < 1e-12
    assert rel_l2(w2.WPx, wake.WPx) < 1e-10 and rel_l2(w2.WPy, wake.WPy) < 1e-10
    assert rel_l2(w2.Z, wake.Z) < 1e-10


@gpu
def test_wake_history_entry_point_rejects_bad_shapes():
    need_gpu()
    from wakis_gb300 import _native as nat
    with pytest.raises(ValueError):
        nat.wake_history(np.zeros((1, 4, 5)), np.zeros((3, 2), np.int32), np.ones(4), 1e3)


# ---------------------------------------------------------------- error mirrors (no GPU)

def test_ezt_argument_without_open_file_raises_like_reference():
    import wakis_gb300 as wg
    w = wg.WakeSolver(save=False, verbose=0, **WAKE)
    w.t, w.zf = np.arange(10) * 1e-12, np.linspace(0, 1e-2, 5)
    with pytest.raises(AttributeError):
        w.calc_long_WP(Ezt=np.zeros((5, 10)))


def test_file_without_slabs_raises_index_error(tmp_path):
    import wakis_gb300 as wg
    meta, _ = synthetic_history(1)
    fname = write_file(tmp_path / "Ez.npz", meta, [])
    w = wg.WakeSolver(save=False, verbose=0, Ez_file=fname, **WAKE)
    with pytest.raises(IndexError):
        w.calc_long_WP_3d()


def test_1d_slabs_in_3d_post_processing_raise_index_error(tmp_path):
    import wakis_gb300 as wg
    meta, slabs = synthetic_history(2, shape3=False, nt=40)
    fname = write_file(tmp_path / "Ez.npz", meta, slabs)
    w = wg.WakeSolver(save=False, verbose=0, Ez_file=fname, **WAKE)
    with pytest.raises(IndexError):
        w.calc_long_WP_3d()


def test_wp_index_equals_oracle_table():
    import wakis_gb300 as wg
    meta, _ = synthetic_history(3, t0=5e-12)
    for skip in (0, 2):
        w = wg.WakeSolver(save=False, verbose=0, skip_cells=skip, **WAKE)
        w.t, w.zf = meta["t"], meta["z"]
        s, it, zz, nz, nt = w._wp_index(300)
        ow = O.OracleWake(skip_cells=skip, **WAKE)
        ow.t, ow.zf = meta["t"], meta["z"]
        s2, it2, valid2, zz2, nt2 = O.wp_index_table(ow, 300)
        np.testing.assert_array_equal(s, s2)
        assert nt == nt2 and nz == it2.shape[1]
        np.testing.assert_array_equal(np.where(it < 0, it + nt, it)[valid2], it2[valid2])
        np.testing.assert_array_equal(it < nt, valid2)


# ---------------------------------------------------------------- pinned to the reference
# tests/golden/wakefile_*.npz: the reference's own WakeSolver.solve() on the seeded
# synthetic Ez files of cases.WAKE_FILE_CASES (tests/golden/make_golden.py)

def _file_case(name, tmp_path):
    case = C.WAKE_FILE_CASES[name]
    meta, slabs = C.synthetic_history(case["seed"], case["nz"], case["nt"], case["shape3"], case["t0"],
                                      case.get("side", 3))
    ref = load_golden(name)
    assert float(ref["slab_sum"]) == float(np.sum(slabs))  # the generator did not drift
    return case, meta, slabs, ref


@pytest.mark.parametrize("name", list(C.WAKE_FILE_CASES))
def test_oracle_file_post_processing_matches_reference(name, tmp_path):
    case, meta, slabs, ref = _file_case(name, tmp_path)
    ow = oracle_wake(meta, slabs, case["plane"], n_transverse_cells=case.get("n_transverse_cells", 1),
                     **case["wake"])
    np.testing.assert_array_equal(ow.s, ref["s"])
    np.testing.assert_array_equal(ow.WP, ref["WP"])
    np.testing.assert_array_equal(ow.f, ref["f"])
    assert rel_l2(ow.Z, ref["Z"]) < 1e-12
    if case["plane"] != "longitudinal":
        np.testing.assert_array_equal(ow.WP_3d, ref["WP_3d"])
        for k in ("WPx", "WPy", "Zx", "Zy"):
            assert rel_l2(getattr(ow, k), ref[k]) < 1e-12, k


@gpu
@pytest.mark.parametrize("name", list(C.WAKE_FILE_CASES))
def test_solve_from_file_matches_reference(name, tmp_path):
    """The device path against the reference's own post-processing of the same file:
    s, WP and WP_3d bit for bit; the transverse wake (prefix sums) and the impedances
    (DFT against numpy's FFT) to FP64 rounding."""
    need_gpu()
    import wakis_gb300 as wg
    case, meta, slabs, ref = _file_case(name, tmp_path)
    fname = write_file(tmp_path / "Ez.npz", meta, slabs)
    w = wg.WakeSolver(save=False, verbose=0, Ez_file=fname, **case["wake"])
    w.n_transverse_cells = case.get("n_transverse_cells", 1)
    w.solve(compute_plane=case["plane"])
    np.testing.assert_array_equal(w.s, ref["s"])
    np.testing.assert_array_equal(w.WP, ref["WP"])
    np.testing.assert_array_equal(w.f, ref["f"])
    assert rel_l2(w.Z, ref["Z"]) < 1e-10
    if case["plane"] != "longitudinal":
        np.testing.assert_array_equal(w.WP_3d, ref["WP_3d"])
        for k in ("WPx", "WPy"):
            assert rel_l2(getattr(w, k), ref[k]) < 1e-12, k
        for k in ("Zx", "Zy"):
            assert rel_l2(getattr(w, k), ref[k]) < 1e-10, k


def test_text_results_round_trip(tmp_path):
    """save_txt / read_txt / load_results follow the reference's file formats
    (wakis/wakeSolver.py:1366-1511): header keys with units, complex columns, lambda.txt."""
    import wakis_gb300 as wg
    w = wg.WakeSolver(save=True, verbose=0, results_folder=str(tmp_path), **WAKE)
    rng = np.random.default_rng(8)
    s = np.linspace(-0.01, 0.02, 50)
    f = np.linspace(0.0, 5e9, 40)
    cols = dict(WP=rng.standard_normal(50), WPx=rng.standard_normal(50), WPy=rng.standard_normal(50),
                lambdas=rng.random(50), Z=rng.standard_normal(40) + 1j * rng.standard_normal(40),
                Zx=rng.standard_normal(40) + 1j * rng.standard_normal(40),
                Zy=rng.standard_normal(40) + 1j * rng.standard_normal(40),
                lambdaf=rng.standard_normal(40) + 1j * rng.standard_normal(40))
    w._savetxt("WP.txt", s, cols["WP"], "WP [V/pC]", "   s [m]")
    w._savetxt("WPx.txt", s, cols["WPx"], "WP [V/pC]", "   s [m]")
    w._savetxt("WPy.txt", s, cols["WPy"], "WP [V/pC]", "   s [m]")
    w._savetxt("lambda.txt", s, cols["lambdas"], "Charge distribution [C/m]", "   s [Hz]")
    w._savetxt("Z.txt", -f, cols["Z"], "Z [Ohm]", "   f [Hz]")
    w._savetxt("spectrum.txt", f, cols["lambdaf"], "Charge distribution spectrum [C/s]", "   f [Hz]")
    w._savetxt("Zx.txt", f, cols["Zx"], "Zx [Ohm]", "   f [Hz]")
    w._savetxt("Zy.txt", f, cols["Zy"], "Zy [Ohm]", "   f [Hz]")
    d = w.read_txt(str(tmp_path / "WP.txt"))
    assert list(d) == ["s[m]", "WP[V/pC]"]
    w2 = wg.WakeSolver(save=False, verbose=0, **WAKE)
    w2.load_results(str(tmp_path))
    np.testing.assert_allclose(w2.s, s, rtol=1e-15)
    np.testing.assert_allclose(w2.f, f, rtol=1e-15)  # abs() of the stored column
    for k, v in cols.items():
        np.testing.assert_allclose(np.asarray(getattr(w2, k)), v, rtol=1e-15, err_msg=k)
    assert w2.wakelength == w2.s[-1] and w2.Ez_file.endswith("/Ez.h5")
    w.save_txt(str(tmp_path / "extra.txt"), s, cols["WP"], x_name="s [m]", y_name="WP [V/pC]")
    assert list(w.read_txt(str(tmp_path / "extra.txt"))) == ["s[m]", "WP[V/pC]"]
