"""Time-dependent sources with the reference's ``update(solver, t)`` protocol
(wakis/sources.py:11-13).

On a wakis_gb300 SolverFIT3D the sources do not write fields from Python every step:
``Beam.update`` arms the beam line current that the E-pass kernel evaluates, and
``PlaneWave`` / ``WavePacket`` provide per-step tables for the device-side hard source
(emsolve).  ``update`` on any other solver-like object writes the fields through their
Field API exactly as the reference does.
"""

import numpy as np
from scipy.constants import c as c_light
from scipy.constants import mu_0


class Beam:
    """Gaussian bunch moving in +z (wakis/sources.py:22-110)."""

    def __init__(self, xsource=0.0, ysource=0.0, beta=1.0, q=1e-9, sigmaz=None, ti=None):
        self.xsource, self.ysource = xsource, ysource
        self.sigmaz = sigmaz
        self.q = q
        self.beta = beta
        self.v = c_light * beta
        if ti is not None:
            self.ti = ti
        else:
            self.ti = 8.548921333333334 * self.sigmaz / self.v
        self.is_first_update = True

    def _first(self, solver):
        self.ixs, self.iys = (np.abs(solver.x - self.xsource).argmin(), np.abs(solver.y - self.ysource).argmin())
        self.zmin = solver.z.min()
        self.is_first_update = False

    @property
    def s0(self):
        return self.zmin - self.v * self.ti

    def vt(self, t):
        """v*t with the reference's scalar types (t may be a numpy float32)."""
        return self.v * t

    def profile_line(self, solver, t):
        """J_z(ixs, iys, :) in FP64 (wakis/sources.py:98-110)."""
        if self.is_first_update:
            self._first(solver)
        s0 = self.zmin - self.v * self.ti
        s = solver.z - self.v * t
        profile = 1 / np.sqrt(2 * np.pi * self.sigmaz ** 2) * np.exp(-((s - s0) ** 2) / (2 * self.sigmaz ** 2))
        return self.q * self.v * profile / solver.dx[self.ixs] / solver.dy[self.iys]

    def update(self, solver, t):
        if self.is_first_update:
            self._first(solver)
        arm = getattr(solver, "_arm_beam", None)
        if arm is not None:
            arm(self, t)
            return
        solver.J[self.ixs, self.iys, :, "z"] = self.profile_line(solver, t)

    def plot(self, t):
        raise NotImplementedError("plotting is not provided")


class PlaneWave:
    """Hard plane-wave source on the plane zs travelling in +z (wakis/sources.py:142-248)."""

    def __init__(self, xs=None, ys=None, zs=0, nodes=None, f=None, amplitude=1.0, beta=1.0, phase=0):
        self.nodes = nodes
        self.beta = beta
        self.xs, self.ys = xs, ys
        self.zs = zs
        self.f = f
        self.amplitude = amplitude
        self.is_first_update = True
        self.phase = phase
        self.vp = self.beta * c_light
        self.w = 2 * np.pi * self.f
        self.kz = self.w / c_light
        self.tmax = np.inf
        if self.nodes is not None:
            self.tmax = self.nodes / self.f

    def _first(self, solver):
        if self.xs is None:
            self.xs = slice(0, solver.Nx)
        if self.ys is None:
            self.ys = slice(0, solver.Ny)
        self.is_first_update = False

    def factors(self, solver, t):
        """(c1, c2, gt) with H_y = c1*g*gt and E_x = c2*g*gt, g = 1."""
        if t <= self.tmax:
            h = -self.amplitude * np.cos(self.w * t + self.phase)
            e = self.amplitude * np.cos(self.w * t + self.phase) / (self.kz / (mu_0 * self.vp))
            return float(h), float(e), 1.0
        return 0.0, 0.0, 1.0

    def profile(self, solver):
        return None

    def update(self, solver, t):
        if self.is_first_update:
            self._first(solver)
        if t <= self.tmax:
            solver.H[self.xs, self.ys, self.zs, "y"] = -self.amplitude * np.cos(self.w * t + self.phase)
            solver.E[self.xs, self.ys, self.zs, "x"] = (self.amplitude * np.cos(self.w * t + self.phase)
                                                        / (self.kz / (mu_0 * self.vp)))
        else:
            solver.H[self.xs, self.ys, self.zs, "y"] = 0.0
            solver.E[self.xs, self.ys, self.zs, "x"] = 0.0

    def plot(self, t):
        raise NotImplementedError("plotting is not provided")


class WavePacket:
    """Hard 2-D Gaussian wave packet on the plane zs travelling in +z
    (wakis/sources.py:285-420)."""

    def __init__(self, xs=None, ys=None, zs=0, sigmaz=None, sigmaxy=None, tinj=None, wavelength=None, f=None,
                 amplitude=1.0, beta=1.0, phase=0):
        self.beta = beta
        self.xs, self.ys = xs, ys
        self.zs = zs
        self.f = f
        self.wavelength = wavelength
        self.sigmaxy = sigmaxy
        self.sigmaz = sigmaz
        self.tinj = tinj
        self.amplitude = amplitude
        self.phase = phase
        if self.f is None:
            self.f = c_light / self.wavelength
        self.w = 2 * np.pi * self.f
        if self.tinj is None:
            self.tinj = 6 * self.sigmaz  # raises TypeError without sigmaz, as the reference does
        self.is_first_update = True

    def _first(self, solver):
        if self.xs is None:
            self.xs = slice(0, solver.Nx)
        if self.ys is None:
            self.ys = slice(0, solver.Ny)
        if self.sigmaz is None:
            self.sigmaz = 10 * np.mean(solver.dz)
        if self.sigmaxy is None:
            self.sigmaxy = 5 * np.mean([np.mean(solver.dx), np.mean(solver.dy)])
        if self.tinj is None:
            self.tinj = 6 * self.sigmaz
        self.is_first_update = False

    def profile(self, solver):
        """gaussxy as assigned to the (xs, ys) block (the reference's meshgrid is 'xy')."""
        if self.is_first_update:
            self._first(solver)
        X, Y = np.meshgrid(solver.x[self.xs], solver.y[self.ys])
        return np.exp(-(X ** 2 + Y ** 2) / (2 * self.sigmaxy ** 2))

    def factors(self, solver, t):
        if self.is_first_update:
            self._first(solver)
        s0 = solver.z.min() - self.tinj
        s = solver.z.min() - self.beta * c_light * t
        gausst = np.exp(-((s - s0) ** 2) / (2 * self.sigmaz ** 2))
        c1 = -self.amplitude * np.cos(self.w * t + self.phase)
        c2 = self.amplitude * mu_0 * c_light * np.cos(self.w * t + self.phase)
        return float(c1), float(c2), float(gausst)

    def update(self, solver, t):
        if self.is_first_update:
            self._first(solver)
        s0 = solver.z.min() - self.tinj
        s = solver.z.min() - self.beta * c_light * t
        X, Y = np.meshgrid(solver.x[self.xs], solver.y[self.ys])
        gaussxy = np.exp(-(X ** 2 + Y ** 2) / (2 * self.sigmaxy ** 2))
        gausst = np.exp(-((s - s0) ** 2) / (2 * self.sigmaz ** 2))
        solver.H[self.xs, self.ys, self.zs, "y"] = (-self.amplitude * np.cos(self.w * t + self.phase) * gaussxy
                                                    * gausst)
        solver.E[self.xs, self.ys, self.zs, "x"] = (self.amplitude * mu_0 * c_light * np.cos(self.w * t + self.phase)
                                                    * gaussxy * gausst)

    def plot(self, t, zmin=0):
        raise NotImplementedError("plotting is not provided")


class _PointSource:
    """Hard source on an index region of one field component: the part Dipole and Pulse
    share (wakis/sources.py:458-762).  ``field`` is 'E', 'H' or 'J', or 'Ex'-style with the
    component; xs, ys, zs are indices or slices and default to the grid centre.  The
    value is written through the solver's Field API every update, so the E / J
    bookkeeping of the solver (explicit J after a J write) applies as for any user write."""

    def __init__(self, field, component, xs, ys, zs, amplitude):
        self.xs, self.ys, self.zs = xs, ys, zs
        self.field = field
        self.component = component
        self.amplitude = amplitude
        if len(field) == 2:
            self.component = field[1]
            self.field = field[0]
        self.is_first_update = True

    def _centre(self, solver):
        if self.xs is None:
            self.xs = int(solver.Nx / 2)
        if self.ys is None:
            self.ys = int(solver.Ny / 2)
        if self.zs is None:
            self.zs = int(solver.Nz / 2)

    def _write(self, solver, value):
        if self.field in ("E", "H", "J"):
            getattr(solver, self.field)[self.xs, self.ys, self.zs, self.component] = value
        else:
            print(f'Field "{self.field}" not valid, should be "E", "H" or "J"]')


class Dipole(_PointSource):
    """Sinusoidal excitation amplitude*sin(w t + phase) (wakis/sources.py:458-565); the
    frequency is nodes / ((z.max - z.min)/c) unless f is given."""

    def __init__(self, field="E", component="z", xs=None, ys=None, zs=None, nodes=10, f=None, amplitude=1.0,
                 phase=0):
        super().__init__(field, component, xs, ys, zs, amplitude)
        self.nodes = nodes
        self.f = f
        self.phase = phase

    def update(self, solver, t):
        if self.is_first_update:
            self._centre(solver)
            if self.f is None:
                T = (solver.z.max() - solver.z.min()) / c_light
                self.f = self.nodes / T
            self.w = 2 * np.pi * self.f
            self.is_first_update = False
        self._write(solver, self.amplitude * np.sin(self.w * t + self.phase))


class Pulse(_PointSource):
    """Pulse of width L (default 50 dt) in x = t*c - delay (wakis/sources.py:567-762):
    'Harris' (four-term cosine window on 0 <= x < L), 'Gaussian' (sigma L/10 centred at
    L/2) or 'Rectangular' (1 on 0 < x < L)."""

    def __init__(self, field="E", component="z", xs=None, ys=None, zs=None, shape="Harris", L=None, amplitude=1.0,
                 delay=0.0):
        super().__init__(field, component, xs, ys, zs, amplitude)
        self.shape = shape
        self.L = L
        self.delay = delay
        profiles = {"harris": self.harris_pulse, "gaussian": self.gaussian_pulse,
                    "rectangular": self.rectangular_pulse}
        self.tprofile = profiles.get(shape.lower())
        if self.tprofile is None:
            print('** shape does not, match available types: "Harris", "Gaussian", "Rectangular"')

    def _harris(self, x):
        return (10 - 15 * np.cos(2 * np.pi / self.L * x) + 6 * np.cos(4 * np.pi / self.L * x)
                - np.cos(6 * np.pi / self.L * x)) / 32

    def harris_pulse(self, t):
        x = t * c_light - self.delay
        if np.ndim(x) > 0:  # time arrays: the window without the cut at L
            return self._harris(x)
        return self._harris(x) if x < self.L else 0.0

    def gaussian_pulse(self, t):
        x = t * c_light - self.delay
        return np.exp(-((x - 5 * (self.L / 10)) ** 2) / (2 * (self.L / 10) ** 2))

    def rectangular_pulse(self, t):
        x = t * c_light - self.delay
        return 1.0 if (x < self.L and x > 0.0) else 0.0

    def update(self, solver, t):
        if self.is_first_update:
            self._centre(solver)
            if self.L is None:
                self.L = 50 * solver.dt
            self.is_first_update = False
        self._write(solver, self.amplitude * self.tprofile(t))
