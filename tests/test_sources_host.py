"""Point sources (Dipole, Pulse; wakis/sources.py:458-762): the product's time profiles
equal the oracle restatement's bit for bit, with the reference's scalar types (a
float32 time from an FP32 solver keeps the Harris window in float32), including the
reference's default pulse width quirk (L = 50*dt in seconds compared with t*c - delay
in metres, so a default-width Harris pulse is zero after the first instant)."""

import numpy as np
import pytest

from oracle import fit_oracle as O
from wakis_gb300 import sources as S


class _Grid:
    Nx, Ny, Nz = 10, 8, 12
    z = np.linspace(-1.0, 1.0, 13)
    dt = np.float32(1.3e-10)


@pytest.mark.parametrize("shape,L,delay", [("Harris", 0.8, 0.0), ("Gaussian", 1.0, 0.05),
                                           ("Rectangular", 0.6, 0.05), ("Harris", None, 0.0)])
@pytest.mark.parametrize("tdtype", [np.float32, np.float64])
def test_pulse_profiles_match_oracle(shape, L, delay, tdtype):
    a = S.Pulse(shape=shape, L=L, delay=delay)
    b = O.OraclePulse(shape=shape, L=L, delay=delay)
    if L is None:
        a.L = b.L = 50 * tdtype(1.3e-10)
    for n in range(40):
        t = n * tdtype(2.1e-10)
        va, vb = a.tprofile(t), b.tprofile(t)
        assert np.asarray(va).dtype == np.asarray(vb).dtype
        assert va == vb or (np.isnan(va) and np.isnan(vb)), (shape, n)


def test_default_width_harris_is_zero_after_start():
    p = S.Pulse(shape="Harris")
    p.L = 50 * np.float32(1.3e-10)
    assert p.tprofile(np.float32(0.0)) == 0.0
    assert all(p.tprofile(n * np.float32(1.3e-10)) == 0.0 for n in range(1, 20))


def test_dipole_defaults_follow_the_grid():
    d = S.Dipole(nodes=3)
    d._centre(_Grid)
    assert (d.xs, d.ys, d.zs) == (5, 4, 6)
    e = S.Dipole(field="Hx")
    assert (e.field, e.component) == ("H", "x")
