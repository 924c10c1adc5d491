"""FieldMonitor (wakis/field_monitors.py): the oracle restatement pinned by the
reference's own unit tests (tests/test_012_field_monitors.py: initial state, one
update, zero-frequency accumulation, the alternating geometric series) and by the
monitor fixtures (tests/golden/monitor_*.npz, the reference's wakesolve with a monitor
attached); the GPU FieldMonitor against the same expectations, the device-loop
epilogue against the Python-loop updates bit for bit, and against the fixtures."""

import numpy as np
import pytest
import torch

import cases as C
from oracle import fit_oracle as O
from oracle_runner import load_golden, rel_l2
from product_runner import run_case

CONST = (1.0, 2.0, 3.0)


def _flat(values, shape):
    n = int(np.prod(shape))
    return np.concatenate([np.full(n, v, dtype=np.float64) for v in values])


# ------------------------------------------------------------------------- oracle (CPU)
def test_oracle_initial_state():
    m = O.OracleFieldMonitor([1.0e9, 2.0e9])
    assert np.allclose(m.frequencies, [1.0e9, 2.0e9]) and m.time_index == 0 and m.dt is None
    assert m.Ex_acc is None and m.shape is None


def test_oracle_single_update_zero_frequency():
    m = O.OracleFieldMonitor([0.0])
    m.update(_flat(CONST, (2, 2, 2)), 1.0e-9, (2, 2, 2))
    assert m.dt == 1.0e-9 and m.shape == (2, 2, 2) and m.time_index == 1
    for acc, v in zip((m.Ex_acc, m.Ey_acc, m.Ez_acc), CONST):
        assert acc.shape == (1, 2, 2, 2) and np.iscomplexobj(acc)
        assert np.allclose(acc[0], v)


def test_oracle_zero_frequency_accumulates_linearly():
    m = O.OracleFieldMonitor([0.0])
    E = _flat((1.0, 0.0, 0.0), (2, 2, 2))
    for _ in range(5):
        m.update(E, 0.1, (2, 2, 2))
    assert m.time_index == 5 and m.dt == 0.1
    assert np.allclose(m.Ex_acc[0], 5.0) and np.allclose(m.Ey_acc, 0.0)


def test_oracle_alternating_phase_sums_to_zero():
    m = O.OracleFieldMonitor([0.5])
    E = _flat((1.0, 0.0, 0.0), (1, 1, 1))
    for _ in range(4):
        m.update(E, 1.0, (1, 1, 1))
    assert np.allclose(m.Ex_acc[0], 0.0, atol=1e-12)


# ------------------------------------------------------------------------- GPU
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")


def _field(values, shape, dtype=np.float64):
    import wakis_gb300 as wg
    f = wg.Field(*shape, dtype=dtype, use_gpu=True)
    f.fromarray(_flat(values, shape).astype(dtype))
    return f


@pytest.mark.gpu
def test_gpu_monitor_matches_reference_unit_tests():
    _gpu()
    import wakis_gb300 as wg
    m = wg.FieldMonitor([1.0e9, 2.0e9])
    assert m.time_index == 0 and m.dt is None and m.get_components()["Ex"] is None
    m = wg.FieldMonitor([0.0])
    f = _field(CONST, (2, 2, 2))
    m.update(f, 1.0e-9)
    comps = m.get_components()
    assert m.shape == (2, 2, 2) and m.time_index == 1 and m.xp is f.xp
    for key, v in zip(("Ex", "Ey", "Ez"), CONST):
        a = comps[key]
        assert tuple(a.shape) == (1, 2, 2, 2) and a.is_complex()
        assert np.allclose(a.cpu().numpy()[0], v)
    m = wg.FieldMonitor([0.5])
    f = _field((1.0, 0.0, 0.0), (1, 1, 1))
    for _ in range(4):
        m.update(f, 1.0)
    assert np.allclose(m.Ex_acc.cpu().numpy()[0], 0.0, atol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_gpu_monitor_update_equals_oracle_bitwise(dtype):
    """Random fields on a 5 x 4 x 3 grid, three frequencies, seven updates: the GPU
    accumulators equal the oracle's (the reference's expression) bit for bit."""
    _gpu()
    import wakis_gb300 as wg
    shape = (5, 4, 3)
    rng = np.random.default_rng(1)
    freqs = [0.0, 1.3e9, 4.7e9]
    dt = dtype(1.7e-12)
    m, o = wg.FieldMonitor(freqs), O.OracleFieldMonitor(freqs)
    for _ in range(7):
        E = rng.standard_normal(3 * 60).astype(dtype)
        f = wg.Field(*shape, dtype=dtype, use_gpu=True)
        f.fromarray(E)
        m.update(f, dt)
        o.update(E, dt, shape)
    for a, b in ((m.Ex_acc, o.Ex_acc), (m.Ey_acc, o.Ey_acc), (m.Ez_acc, o.Ez_acc)):
        np.testing.assert_array_equal(a.cpu().numpy(), b)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["monitor_f64", "monitor_f32"])
def test_device_loop_monitor_equals_python_loop(name, tmp_path, monkeypatch):
    """wakesolve with the monitor as a device-loop epilogue equals the Python step loop
    calling FieldMonitor.update after each step (two-pass kernels in both: bit for bit),
    and the default (fused) device loop agrees to rounding."""
    _gpu()
    monkeypatch.setenv("WAKIS_GB300_KERNELS", "direct")
    dev = run_case(name, tmpdir=tmp_path)
    loop = run_case(name, tmpdir=tmp_path, userloop_wake=True)
    for k in ("Ex_acc", "Ey_acc", "Ez_acc", "WP", "Z", "E"):
        np.testing.assert_array_equal(dev[k], loop[k], err_msg=k)
    monkeypatch.setenv("WAKIS_GB300_KERNELS", "auto")
    fused = run_case(name, tmpdir=tmp_path)
    tol = 1e-12 if C.CASES[name]["dtype"] == "float64" else 1e-5
    for k in ("Ex_acc", "Ey_acc", "Ez_acc"):
        assert rel_l2(fused[k], dev[k]) < tol, k
    g = load_golden(name)
    ftol = 1e-10 if C.CASES[name]["dtype"] == "float64" else 1e-3
    for k in ("Ex_acc", "Ey_acc", "Ez_acc"):
        assert rel_l2(fused[k], g[k]) < ftol, (k, rel_l2(fused[k], g[k]))
