"""Host-side logic of the serving loop (no GPU): request generation, footprints,
admission policy, and the pool entry points' argument checks."""

import ctypes as C

import numpy as np
import pytest

import wakis_gb300._native as nat
from wakis_gb300 import serving as S


def test_cavity_sweep_requests_are_seeded_and_in_range():
    a = S.cavity_sweep_requests(64, seed=3)
    b = S.cavity_sweep_requests(64, seed=3)
    assert [dataclass_tuple(r) for r in a] == [dataclass_tuple(r) for r in b]
    assert len(a) == 64 and [r.tag for r in a] == list(range(64))
    for r in a:
        assert 20e-3 <= r.side <= 60e-3
        assert 3e-3 <= r.rp <= 8e-3
        assert 48 <= r.n <= 160
        assert 5e-3 <= r.sigmaz <= 15e-3
        assert r.sigma == 0.0 or 1e3 <= r.sigma <= 1e6
        assert r.arrival == 0.0
        assert r.cells == 2 * r.n ** 3
    assert 10 < sum(r.lossy for r in a) < 54
    c = S.cavity_sweep_requests(64, seed=3, rate_hz=2.0)
    t = np.array([r.arrival for r in c])
    assert np.all(np.diff(t) > 0)
    # same instances, only the arrival times are added
    assert [(r.side, r.n, r.sigma) for r in c] != [] and c[0].arrival > 0


def dataclass_tuple(r):
    return (r.tag, r.side, r.rp, r.n, r.sigmaz, r.sigma, r.arrival, r.wakelength)


def test_footprint_counts_fields_materials_and_coefficients():
    r = S.CavityRequest(tag=0, side=0.04, rp=0.005, n=100, sigmaz=0.01, sigma=0.0)
    N = r.cells
    f32 = S.footprint_bytes(r, np.float32)
    assert f32 == N * (36 + 72 + 24 + 1 + 2) + 8 * 2 ** 20  # ... + mask byte + 2-byte coefficient code
    lossy = S.CavityRequest(tag=1, side=0.04, rp=0.005, n=100, sigmaz=0.01, sigma=1e4)
    assert S.footprint_bytes(lossy, np.float32) - f32 == 12 * N
    assert S.footprint_bytes(r, np.float64) > f32


def test_cfl_dt_follows_the_solver_formula():
    from scipy.constants import c
    r = S.CavityRequest(tag=0, side=0.03, rp=0.005, n=60, sigmaz=0.01, sigma=0.0)
    d = 1.2 * r.side / r.n
    dt = 1.0 / (c * np.sqrt(3 / d ** 2))
    assert S.cfl_dt(r, np.float64) == pytest.approx(dt, rel=1e-12)
    assert S.cfl_dt(r, np.float32) == float(np.float32(S.cfl_dt(r, np.float64)))
    lossy = S.CavityRequest(tag=0, side=0.03, rp=0.005, n=60, sigmaz=0.01, sigma=1e5)
    assert S.cfl_dt(lossy, np.float64) == pytest.approx(dt / 2, rel=1e-12)


class _Budget:
    def __init__(self, free):
        self.free = free

    def reserve(self, b):
        if b <= self.free:
            self.free -= b
            return True
        return False


def test_admission_first_fit_in_arrival_order():
    sizes = {0: 10, 1: 3, 2: 3, 3: 4, 4: 1}
    q = [0, 1, 2, 3, 4]
    a = S.Admission(max_bypass=8)
    bud = _Budget(8)
    got = list(a.admit(q, sizes.get, bud.reserve))
    assert [r for r, _ in got] == [1, 2, 4]
    assert q == [0, 3]
    assert bud.free == 1


def test_admission_bypass_limit_protects_the_oldest_request():
    sizes = {0: 10, 1: 1, 2: 1, 3: 1, 4: 1}
    q = [0, 1, 2, 3, 4]
    a = S.Admission(max_bypass=2)
    bud = _Budget(5)
    got = [r for r, _ in a.admit(q, sizes.get, bud.reserve)]
    assert got == [1, 2]  # two bypasses, then only the head may go
    assert q == [0, 3, 4]
    assert [r for r, _ in a.admit(q, sizes.get, bud.reserve)] == []
    bud.free = 10
    assert [r for r, _ in a.admit(q, sizes.get, bud.reserve)] == [0]
    # a new head resets the count
    bud.free = 2
    assert [r for r, _ in a.admit(q, sizes.get, bud.reserve)] == [3, 4]


def test_poisson_rate_makes_the_queue_grow():
    reqs = S.cavity_sweep_requests(16, seed=3)
    rate = S.poisson_rate_for(reqs, 4 << 30, service_rate_cells_per_s=50e9, load=1.5)
    work = np.mean([r.cells * S._steps_estimate(r) for r in reqs])
    assert rate == pytest.approx(1.5 * 50e9 / work)
    assert rate > 0


def test_pool_entry_points_check_arguments_without_a_device():
    lib = nat.load()
    assert lib.fit_pool_reserve(None, 10) == -1
    assert lib.fit_pool_release(None, 10) == -1
    assert lib.fit_pool_submit(None, None, 0, 1, 0) == -1
    assert lib.fit_pool_poll(None, None, 0, 0) == -1
    assert lib.fit_pool_stats(None, None) == -1
    assert lib.fit_pool_destroy(None) == 0
    h = C.c_void_p()
    assert lib.fit_pool_create(0, 0, 64, 0, C.byref(h)) == -1          # no budget
    assert lib.fit_pool_create(0, 1 << 30, 0, 0, C.byref(h)) == -1     # chunk out of range
    assert lib.fit_pool_create(0, 1 << 30, 64, 99, C.byref(h)) == -1   # ctas_per_sm out of range
    buf = C.create_string_buffer(256)
    lib.fit_pool_last_error(None, buf, 256)
    assert b"ctas_per_sm" in buf.value


def test_pool_without_a_device_raises():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    with pytest.raises(nat.FitError) as e:
        nat.Pool(1 << 30)
    assert e.value.code == -6
