"""GPU parity: the CUDA path (wakis_gb300 through libwakis_fit.so) against the CPU oracle
and the reference fixtures, on every case of tests/golden/cases.py.

Tolerances: FP64 cases 1e-10 relative L2 (fields, WP, WP_3d, Z); FP32 cases 1e-4 relative
L2 on WP / Z and 1e-3 on the raw fields (different rounding order of the same FP32
arithmetic); transverse wakes of symmetric cases (~0) are compared on the scale of
WP / Z.  Index sets (s, f, Nt, dt) must be identical."""

import numpy as np
import pytest
import torch

import cases as C
from oracle_runner import load_golden, rel_l2, run_oracle_case
from product_runner import run_case

pytestmark = pytest.mark.gpu

FIELD_TOL = {"float64": 1e-10, "float32": 1e-3}
WAKE_TOL = {"float64": 1e-10, "float32": 1e-4}


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")


def _err(a, b, scale_ref=None):
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    scale = float(np.linalg.norm(b))
    if scale_ref is not None:
        scale = max(scale, 1e-3 * float(np.linalg.norm(np.asarray(scale_ref, dtype=np.complex128))))
    return float(np.linalg.norm(a - b)) / max(scale, 1e-300)


def _compare(name, got, ref, what):
    case = C.CASES[name]
    dt = case["dtype"]
    for k, v in ref.items():
        if k not in got:
            continue
        if k == "Nt":
            assert int(got[k]) == int(v), f"{what} {name}: Nt"
        elif k == "dt":
            assert got[k] == v, f"{what} {name}: dt {got[k]} != {v}"
        elif k in ("s", "f"):
            np.testing.assert_array_equal(got[k], v, err_msg=f"{what} {name}: {k}")
        elif k in ("E", "H", "J", "probes", "Ey") or k.endswith("_acc"):
            e = _err(got[k], v)
            assert e <= FIELD_TOL[dt], f"{what} {name}: {k} rel L2 {e:.3e}"
        elif k in ("WPx", "WPy"):
            e = _err(got[k], v, ref["WP"])
            assert e <= WAKE_TOL[dt], f"{what} {name}: {k} rel L2 {e:.3e}"
        elif k in ("Zx", "Zy"):
            e = _err(got[k], v, ref["Z"])
            assert e <= WAKE_TOL[dt], f"{what} {name}: {k} rel L2 {e:.3e}"
        else:
            e = _err(got[k], v)
            assert e <= WAKE_TOL[dt], f"{what} {name}: {k} rel L2 {e:.3e}"


@pytest.mark.parametrize("name", list(C.CASES))
def test_case_vs_reference_and_oracle(name, tmp_path):
    got = run_case(name, tmpdir=tmp_path)
    _compare(name, got, load_golden(name), "vs reference fixture")
    _compare(name, got, run_oracle_case(name), "vs oracle")


def test_wavepacket_device_loop_matches_step_loop(tmp_path):
    """The same wave-packet run through the device loop (no callback) and the Python
    step loop (callback) ends in the same fields, equal to the reference's."""
    case = dict(C.CASES["wavepacket_f64"])
    case.pop("probes")
    got = run_case("wavepacket_f64", case=case, tmpdir=tmp_path)
    ref = load_golden("wavepacket_f64")
    for k in ("E", "H"):
        assert _err(got[k], ref[k]) <= 1e-10, k


def test_planewave_step_loop_matches_device_loop(tmp_path):
    """The plane-wave run through the Python step loop (a callback forces it) ends in the
    fields of the device loop and of the reference."""
    case = dict(C.CASES["planewave_f32"])
    case["probes"] = 2
    case["probe_margin"] = 0
    got = run_case("planewave_f32", case=case, tmpdir=tmp_path)
    ref = load_golden("planewave_f32")
    for k in ("E", "H"):
        assert _err(got[k], ref[k]) <= 1e-3, k


@pytest.mark.parametrize("name", ["lossy_f32", "cavity_f64", "mixed_bc_f64", "pmc_beam_f64"])
def test_staged_kernels_match_direct_kernels(name, tmp_path, monkeypatch):
    """The persistent bulk-copy kernels and the direct-load kernels run the same
    arithmetic: fields and wakes agree bit for bit."""
    import wakis_gb300.solverFIT3D as sf
    orig = sf.SolverFIT3D._sync_coeffs
    out = []
    for staged in (1, 0):
        def patched(self, _o=orig, _s=staged):
            self._ctx.call("fit_set_kernel_variant", _s)
            _o(self)
        monkeypatch.setattr(sf.SolverFIT3D, "_sync_coeffs", patched)
        out.append(run_case(name, tmpdir=tmp_path))
    monkeypatch.setattr(sf.SolverFIT3D, "_sync_coeffs", orig)
    for k in ("E", "H", "J", "WP", "Z"):
        if k in out[0]:
            np.testing.assert_array_equal(out[0][k], out[1][k], err_msg=k)


def test_wake_step_loop_matches_device_loop(tmp_path):
    """wakesolve with a callback (Python step loop) equals the graph-replayed loop."""
    import wakis_gb300 as wg
    from product_runner import make_grid, make_solver
    case = C.CASES["lossy_f64"]
    out = []
    for use_cb in (False, True):
        grid = make_grid(wg, case)
        wake = wg.WakeSolver(wakelength=case["wakelength"], save=False, verbose=0, results_folder=str(tmp_path),
                             **case["wake"])
        s = make_solver(wg, case, grid, wake)
        cb = (lambda sv, t: None) if use_cb else None
        s.wakesolve(wakelength=case["wakelength"], callback=cb)
        out.append((wake.WP.copy(), wake.Z.copy(), s.E.numpy()))
    assert rel_l2(out[0][0], out[1][0]) < 1e-13
    assert rel_l2(out[0][2], out[1][2]) < 1e-13
