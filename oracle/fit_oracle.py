"""CPU oracle for the FIT leapfrog path of Wakis -- TEST INFRASTRUCTURE ONLY.

This module is a numpy/scipy restatement of the reference's algorithm for the hot
path (grid metrics, boundary handling, materials, PML, time step, the sparse-matrix
leapfrog step, the beam / plane-wave sources, the wakesolve / emsolve drivers and the
wake-potential / impedance post-processing).  It is the reference the parity tests
compare the CUDA path against, and the CPU baseline that ``bench.py`` times.  Only
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline / reference
legs may import it; the product package ``wakis_gb300`` never does.

Pinning: every function is checked by ``tests/test_oracle_golden.py`` against
fixtures generated by running the reference itself (``tests/golden/make_golden.py``)
and against the golden vectors held by the reference's own ``test_001``.

Citations are ``path:line`` inside the reference project (Wakis 0.7.0).
The operator is held as scipy CSR matrices exactly as the reference assembles it,
so the arithmetic (association order of the diagonal products, dtype of every
intermediate) follows the reference.
"""

import numpy as np
from scipy.constants import c as c_light
from scipy.constants import epsilon_0 as eps_0
from scipy.constants import mu_0
from scipy.sparse import bmat, diags

MATERIAL_LIB = {  # wakis/materials.py:28-41
    "pec": [np.inf, 1.0],
    "vacuum": [1.0, 1.0],
    "dielectric": [10.0, 1.0],
    "lossy metal": [10, 1.0, 10],
    "copper": [5.8e07, 1.0, 5.8e07],
    "berillium": [2.5e07, 1.0, 2.5e07],
    "stainless steel": [1.4e06, 1.0, 1.4e06],
}

PEC_LIKE = ("electric", "pec", "pml")


# --------------------------------------------------------------------------------------
# flat-array helpers: a component is stored in Fortran order n = i + Nx*j + Nx*Ny*k
# (wakis/field.py:22-24,139-168)
# --------------------------------------------------------------------------------------
def comp_view(arr, N, shape, d):
    """(Nx,Ny,Nz) Fortran-order view of component d of a flat 3N array."""
    return arr[d * N:(d + 1) * N].reshape(shape, order="F")


# --------------------------------------------------------------------------------------
# grid metrics: wakis/gridFIT3D.py:263-305
# --------------------------------------------------------------------------------------
class OracleGrid:
    def __init__(self, x, y, z):
        self.x, self.y, self.z = np.asarray(x, float), np.asarray(y, float), np.asarray(z, float)
        self.Nx, self.Ny, self.Nz = len(self.x) - 1, len(self.y) - 1, len(self.z) - 1
        self.N = self.Nx * self.Ny * self.Nz
        self.shape = (self.Nx, self.Ny, self.Nz)
        self.dx, self.dy, self.dz = np.diff(self.x), np.diff(self.y), np.diff(self.z)
        X, Y, Z = np.meshgrid(self.x, self.y, self.z, indexing="ij")
        Lx = X[1:, 1:, 1:] - X[:-1, :-1, :-1]
        Ly = Y[1:, 1:, 1:] - Y[:-1, :-1, :-1]
        Lz = Z[1:, 1:, 1:] - Z[:-1, :-1, :-1]
        self.L = self._flat(Lx, Ly, Lz)
        self.iA = self._flat(np.divide(1.0, Ly * Lz), np.divide(1.0, Lx * Lz), np.divide(1.0, Lx * Ly))
        tx = (self.x[1:] + self.x[:-1]) / 2
        ty = (self.y[1:] + self.y[:-1]) / 2
        tz = (self.z[1:] + self.z[:-1]) / 2
        tx, ty, tz = np.append(tx, tx[-1]), np.append(ty, ty[-1]), np.append(tz, tz[-1])
        tX, tY, tZ = np.meshgrid(tx, ty, tz, indexing="ij")
        tLx = tX[1:, 1:, 1:] - tX[:-1, :-1, :-1]
        tLy = tY[1:, 1:, 1:] - tY[:-1, :-1, :-1]
        tLz = tZ[1:, 1:, 1:] - tZ[:-1, :-1, :-1]
        self.tL = self._flat(tLx, tLy, tLz)

        def safe_inv(a):
            return np.divide(1.0, a, out=np.zeros_like(a), where=a != 0)

        self.itA = self._flat(safe_inv(tLy * tLz), safe_inv(tLx * tLz), safe_inv(tLx * tLy))
        # cell centres, as SolverFIT3D exposes them (wakis/solverFIT3D.py:161-163)
        self.xc = self.x[:-1] + self.dx / 2
        self.yc = self.y[:-1] + self.dy / 2
        self.zc = self.z[:-1] + self.dz / 2

    def _flat(self, a, b, c):
        return np.concatenate([m.reshape(-1, order="F") for m in (a, b, c)])

    def comp(self, arr, d):
        return comp_view(arr, self.N, self.shape, d)


def uniform_grid(xmin, xmax, ymin, ymax, zmin, zmax, Nx, Ny, Nz):
    """wakis/gridFIT3D.py:161-169 (domain extents + cell counts)."""
    return OracleGrid(np.linspace(xmin, xmax, Nx + 1), np.linspace(ymin, ymax, Ny + 1),
                      np.linspace(zmin, zmax, Nz + 1))


# --------------------------------------------------------------------------------------
# boundary conditions: wakis/boundaries.py:14-188
# --------------------------------------------------------------------------------------
def face_mask(g, values, dtype=np.int8):
    """Tangential face mask, last write wins in the order x-lo, x-hi, y-lo, y-hi,
    z-lo, z-hi (wakis/boundaries.py:90-101)."""
    xlo, xhi, ylo, yhi, zlo, zhi = values
    BC = np.ones(3 * g.N, dtype=dtype)
    for di, d in enumerate("xyz"):
        m = g.comp(BC, di)
        if d != "x":
            m[0, :, :] = xlo
            m[-1, :, :] = xhi
        if d != "y":
            m[:, 0, :] = ylo
            m[:, -1, :] = yhi
        if d != "z":
            m[:, :, 0] = zlo
            m[:, :, -1] = zhi
    return BC


def apply_bcs(g, bc_low, bc_high):
    """Returns dict(tL, itA, Dpec, Dpmc, activate_abc, activate_pml).

    tL / itA are edited copies (periodic: wakis/boundaries.py:36-70; abc high faces:
    wakis/boundaries.py:153-181).  Dpec multiplies columns of C (wakis/boundaries.py:73-110),
    Dpmc multiplies rows (wakis/boundaries.py:113-150).  As in the reference the PMC
    block starts from the face values left by the PEC block.
    """
    lo = [b.lower() for b in bc_low]
    hi = [b.lower() for b in bc_high]
    tL, itA, L, iA = g.tL.copy(), g.itA.copy(), g.L, g.iA
    c = g.comp

    def wrap(axis):
        if axis == 0:
            c(tL, 0)[-1, :, :] = c(L, 0)[0, :, :]
            c(itA, 1)[-1, :, :] = c(iA, 1)[0, :, :]
            c(itA, 2)[-1, :, :] = c(iA, 2)[0, :, :]
        elif axis == 1:
            c(tL, 1)[:, -1, :] = c(L, 1)[:, 0, :]
            c(itA, 0)[:, -1, :] = c(iA, 0)[:, 0, :]
            c(itA, 2)[:, -1, :] = c(iA, 2)[:, 0, :]
        else:
            c(tL, 2)[:, :, -1] = c(L, 2)[:, :, 0]
            c(itA, 0)[:, :, -1] = c(iA, 0)[:, :, 0]
            c(itA, 1)[:, :, -1] = c(iA, 1)[:, :, 0]

    if "periodic" in lo:
        for a in range(3):
            if lo[a] == "periodic" and hi[a] == "periodic":
                wrap(a)
    vals = [1.0] * 6  # xlo, xhi, ylo, yhi, zlo, zhi
    Dpec = Dpmc = None
    if any(b in PEC_LIKE for b in lo) or any(b in PEC_LIKE for b in hi):
        for a in range(3):
            if lo[a] in PEC_LIKE:
                vals[2 * a] = 0
            if hi[a] in PEC_LIKE:
                vals[2 * a + 1] = 0
        Dpec = face_mask(g, vals)
    if any(b in ("magnetic", "pmc") for b in lo) or any(b in ("magnetic", "pmc") for b in hi):
        # the reference tests `.lower() == "magnetic"` or the raw string == "pmc"
        for a in range(3):
            if lo[a] == "magnetic" or bc_low[a] == "pmc":
                vals[2 * a] = 0
            if hi[a] == "magnetic" or bc_high[a] == "pmc":
                vals[2 * a + 1] = 0
        Dpmc = face_mask(g, vals)
    activate_abc = "abc" in lo or "abc" in hi
    if activate_abc:
        for a in range(3):
            if hi[a] == "abc":
                wrap(a)
    activate_pml = "pml" in lo or "pml" in hi
    return dict(tL=tL, itA=itA, Dpec=Dpec, Dpmc=Dpmc, activate_abc=activate_abc,
                activate_pml=activate_pml)


# --------------------------------------------------------------------------------------
# materials: wakis/solverFIT3D.py:240-279,438-502 ; PML: wakis/boundaries.py:190-305
# --------------------------------------------------------------------------------------
def build_materials(g, bg, solids, use_sibc, dtype):
    """solids: list of (mask (Nx,Ny,Nz) bool, material list or library key)."""
    if isinstance(bg, str):
        bg = MATERIAL_LIB[bg.lower()]
    use_conductivity = False
    if len(bg) == 3:
        eps_bg, mu_bg, sigma_bg = bg[0] * eps_0, bg[1] * mu_0, bg[2]
        use_conductivity = True
    else:
        eps_bg, mu_bg, sigma_bg = bg[0] * eps_0, bg[1] * mu_0, 0.0
    with np.errstate(divide="ignore"):
        ieps = np.ones(3 * g.N, dtype=dtype) * (1.0 / eps_bg)
        imu = np.ones(3 * g.N, dtype=dtype) * (1.0 / mu_bg)
    sigma = np.ones(3 * g.N, dtype=dtype) * sigma_bg
    for mask, mat in solids:
        if isinstance(mat, str):
            mat = MATERIAL_LIB[mat.lower()]
        m = np.asarray(mask).astype(int)
        eps = mat[0] * eps_0
        mu = mat[1] * mu_0
        if len(mat) == 3:
            sig = mat[2]
            if use_sibc and sig > 0.0:
                eps = sig * eps_0  # relaxation-time form (wakis/solverFIT3D.py:470-472)
            for d in range(3):
                s = g.comp(sigma, d)
                s[...] = (s + s * (-1.0 * m)).astype(dtype)
                s[...] = (s + m * sig).astype(dtype)
            use_conductivity = True
        elif sigma_bg > 0.0:
            for d in range(3):
                s = g.comp(sigma, d)
                s[...] = (s + s * (-1.0 * m)).astype(dtype)
        with np.errstate(divide="ignore"):
            for arr, val in ((ieps, eps), (imu, mu)):
                for d in range(3):
                    a = g.comp(arr, d)
                    a[...] = (a + a * (-1.0 * m)).astype(dtype)
                for d in range(3):
                    a = g.comp(arr, d)
                    a[...] = (a + m * 1.0 / val).astype(dtype)
    return ieps, imu, sigma, use_conductivity


def apply_pml(g, ieps, sigma, bc_low, bc_high, n_pml):
    """Graded-conductivity PML slabs (wakis/boundaries.py:190-305): inside each slab
    ieps = 1/eps0 and sigma = geomspace(1.0 -> 5e-3) with the outermost cell = 1.0;
    slabs are written x-lo, y-lo, z-lo, x-hi, y-hi, z-hi."""
    lo = [b.lower() for b in bc_low]
    hi = [b.lower() for b in bc_high]
    prof_lo = np.geomspace(1.0, 5.0e-3, n_pml)
    prof_hi = np.geomspace(5.0e-3, 1.0, n_pml)
    for a in range(3):
        if lo[a] == "pml":
            for d in range(3):
                ie, sg = g.comp(ieps, d), g.comp(sigma, d)
                for i in range(n_pml):
                    sl = [slice(None)] * 3
                    sl[a] = i
                    ie[tuple(sl)] = 1 / eps_0
                    sg[tuple(sl)] = 0.0 + 1 * prof_lo[i]
    for a in range(3):
        if hi[a] == "pml":
            for d in range(3):
                ie, sg = g.comp(ieps, d), g.comp(sigma, d)
                for i in range(1, n_pml + 1):
                    sl = [slice(None)] * 3
                    sl[a] = -i
                    ie[tuple(sl)] = 1 / eps_0
                    sg[tuple(sl)] = 0.0 + 1 * prof_hi[-i]


def timestep(g, cfln, dt, dtype, use_conductivity, ieps, sigma):
    """wakis/solverFIT3D.py:294-318."""
    if dt is None:
        dt = cfln / (c_light * np.sqrt(1 / np.min(g.dx) ** 2 + 1 / np.min(g.dy) ** 2
                                       + 1 / np.min(g.dz) ** 2))
    dt = dtype(dt)
    if use_conductivity:
        mask = np.logical_and(sigma != 0, ieps != 0)
        tau = (1 / ieps[mask]) / sigma[mask]
        if dt > tau.min():  # an empty mask raises, as in the reference
            dt = tau.min()
    return dt


# --------------------------------------------------------------------------------------
# the solver: operator assembly wakis/solverFIT3D.py:203-227,337-344 ;
# step wakis/solverFIT3D.py:504-525 ; ghosts wakis/solverFIT3D.py:842-862
# --------------------------------------------------------------------------------------
class OracleSolver:
    def __init__(self, grid, bc_low, bc_high, solids=(), bg=(1.0, 1.0), use_sibc=True,
                 cfln=0.5, dt=None, dtype=np.float64, n_pml=10):
        g = self.grid = grid
        self.dtype = dtype
        self.Nx, self.Ny, self.Nz, self.N = g.Nx, g.Ny, g.Nz, g.N
        self.x, self.y, self.z = g.xc, g.yc, g.zc
        self.dx, self.dy, self.dz = g.dx, g.dy, g.dz
        self.bc_low, self.bc_high = list(bc_low), list(bc_high)
        bc = apply_bcs(g, bc_low, bc_high)
        self.activate_abc, self.activate_pml = bc["activate_abc"], bc["activate_pml"]
        ieps, imu, sigma, use_cond = build_materials(g, list(bg) if not isinstance(bg, str) else bg,
                                                     solids, use_sibc, dtype)
        self.use_conductivity = use_cond or self.activate_pml
        if self.activate_pml:
            apply_pml(g, ieps, sigma, bc_low, bc_high, n_pml)
        self.ieps, self.imu, self.sigma = ieps, imu, sigma
        self.dt = timestep(g, cfln, dt, dtype, self.use_conductivity, ieps, sigma)
        N = self.N
        Px = diags([-1, 1], [0, 1], shape=(N, N), dtype=np.int8)
        Py = diags([-1, 1], [0, g.Nx], shape=(N, N), dtype=np.int8)
        Pz = diags([-1, 1], [0, g.Nx * g.Ny], shape=(N, N), dtype=np.int8)
        C = bmat([[None, -Pz, Py], [Pz, None, -Px], [-Py, Px, None]], format="csc", dtype=np.int8)
        if bc["Dpec"] is not None:
            C = C @ diags(bc["Dpec"], dtype=np.int8)
        if bc["Dpmc"] is not None:
            C = diags(bc["Dpmc"], dtype=np.int8) @ C
        Ds = diags(g.L, dtype=dtype)
        iDa = diags(g.iA, dtype=dtype)
        tDs = diags(bc["tL"], dtype=dtype)
        itDa = diags(bc["itA"], dtype=dtype)
        iDeps = diags(ieps, dtype=dtype)
        iDmu = diags(imu, dtype=dtype)
        self.M_H = (((iDa @ iDmu) @ C) @ Ds).tocsr()
        self.M_E = (((iDeps @ itDa) @ C.transpose()) @ tDs).tocsr()
        self.E = np.zeros(3 * N, dtype=dtype)
        self.H = np.zeros(3 * N, dtype=dtype)
        self.J = np.zeros(3 * N, dtype=dtype)
        self.step_0 = True

    def comp(self, arr, d):
        return self.grid.comp(arr, d)

    def set_ghosts_to_0(self):
        for d in range(3):
            h = self.comp(self.H, d)
            if d != 0:
                h[-1, :, :] = 0.0
            if d != 1:
                h[:, -1, :] = 0.0
            if d != 2:
                h[:, :, -1] = 0.0
        self.comp(self.E, 0)[-1, :, :] = 0.0
        self.comp(self.E, 1)[:, -1, :] = 0.0
        self.comp(self.E, 2)[:, :, -1] = 0.0

    def one_step(self):
        if self.step_0:
            self.set_ghosts_to_0()
            self.step_0 = False
        self.H[:] = self.H - (self.dt * self.M_H) @ self.E
        self.E[:] = self.E + self.dt * (self.M_E @ self.H - self.ieps * self.J)
        if self.use_conductivity:
            self.J[:] = self.sigma * self.E

    # ABC first-order extrapolation as emsolve applies it on the CPU
    # (wakis/routines.py:183-220, wakis/boundaries.py:307-404): the snapshots are live
    # views, so every low ABC face copies the current index-1 plane; high faces are
    # no-ops; x, y, z in that order.
    def abc_update(self):
        lo = [b.lower() for b in self.bc_low]
        hi = [b.lower() for b in self.bc_high]
        for a in range(3):
            if lo[a] == "abc" and hi[a] == "abc":
                raise KeyError("xyz"[a] + "lo")
        for a in range(3):
            if lo[a] == "abc":
                for arr in (self.E, self.H):
                    for d in range(3):
                        v = self.comp(arr, d)
                        sl0 = [slice(None)] * 3
                        sl1 = [slice(None)] * 3
                        sl0[a], sl1[a] = 0, 1
                        v[tuple(sl0)] = v[tuple(sl1)]


# --------------------------------------------------------------------------------------
# sources: wakis/sources.py:22-110 (Beam), 142-248 (PlaneWave), 285-420 (WavePacket)
# --------------------------------------------------------------------------------------
class OracleBeam:
    def __init__(self, xsource=0.0, ysource=0.0, beta=1.0, q=1e-9, sigmaz=None, ti=None):
        self.xsource, self.ysource = xsource, ysource
        self.sigmaz, self.q, self.beta = sigmaz, q, beta
        self.v = c_light * beta
        self.ti = ti if ti is not None else 8.548921333333334 * self.sigmaz / self.v
        self.first = True

    def profile_line(self, solver, t):
        if self.first:
            self.ixs = np.abs(solver.x - self.xsource).argmin()
            self.iys = np.abs(solver.y - self.ysource).argmin()
            self.zmin = solver.z.min()
            self.first = False
        s0 = self.zmin - self.v * self.ti
        s = solver.z - self.v * t
        profile = 1 / np.sqrt(2 * np.pi * self.sigmaz ** 2) * np.exp(-((s - s0) ** 2) / (2 * self.sigmaz ** 2))
        return self.q * self.v * profile / solver.dx[self.ixs] / solver.dy[self.iys]

    def update(self, solver, t):
        line = self.profile_line(solver, t)
        solver.comp(solver.J, 2)[self.ixs, self.iys, :] = line


class OraclePlaneWave:
    def __init__(self, xs=None, ys=None, zs=0, nodes=None, f=None, amplitude=1.0, beta=1.0, phase=0):
        self.xs, self.ys, self.zs = xs, ys, zs
        self.f, self.amplitude, self.beta, self.phase = f, amplitude, beta, phase
        self.vp = beta * c_light
        self.w = 2 * np.pi * f
        self.kz = self.w / c_light
        self.tmax = np.inf if nodes is None else nodes / f

    def update(self, solver, t):
        xs = self.xs if self.xs is not None else slice(0, solver.Nx)
        ys = self.ys if self.ys is not None else slice(0, solver.Ny)
        hy, ex = solver.comp(solver.H, 1), solver.comp(solver.E, 0)
        if t <= self.tmax:
            hy[xs, ys, self.zs] = -self.amplitude * np.cos(self.w * t + self.phase)
            ex[xs, ys, self.zs] = self.amplitude * np.cos(self.w * t + self.phase) / (self.kz / (mu_0 * self.vp))
        else:
            hy[xs, ys, self.zs] = 0.0
            ex[xs, ys, self.zs] = 0.0


class OracleWavePacket:
    def __init__(self, xs=None, ys=None, zs=0, sigmaz=None, sigmaxy=None, tinj=None,
                 wavelength=None, f=None, amplitude=1.0, beta=1.0, phase=0):
        self.xs, self.ys, self.zs = xs, ys, zs
        self.sigmaz, self.sigmaxy, self.tinj = sigmaz, sigmaxy, tinj
        self.amplitude, self.beta, self.phase = amplitude, beta, phase
        self.f = f if f is not None else c_light / wavelength
        self.w = 2 * np.pi * self.f
        if self.tinj is None and self.sigmaz is not None:
            self.tinj = 6 * self.sigmaz
        self.first = True

    def update(self, solver, t):
        if self.first:
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
            self.first = False
        s0 = solver.z.min() - self.tinj
        s = solver.z.min() - self.beta * c_light * t
        X, Y = np.meshgrid(solver.x[self.xs], solver.y[self.ys])
        gaussxy = np.exp(-(X ** 2 + Y ** 2) / (2 * self.sigmaxy ** 2))
        gausst = np.exp(-((s - s0) ** 2) / (2 * self.sigmaz ** 2))
        hy, ex = solver.comp(solver.H, 1), solver.comp(solver.E, 0)
        hy[self.xs, self.ys, self.zs] = -self.amplitude * np.cos(self.w * t + self.phase) * gaussxy * gausst
        ex[self.xs, self.ys, self.zs] = (self.amplitude * mu_0 * c_light * np.cos(self.w * t + self.phase)
                                         * gaussxy * gausst)


# --------------------------------------------------------------------------------------
# drivers: wakis/routines.py:17-229 (emsolve) and 231-485 (wakesolve)
# --------------------------------------------------------------------------------------
class _OraclePointSource:
    """Hard source on an index region of one field component (wakis/sources.py:458-762:
    the common part of Dipole and Pulse).  'Ex'-style field names carry the component;
    regions default to the grid centre."""

    def __init__(self, field, component, xs, ys, zs, amplitude):
        self.xs, self.ys, self.zs = xs, ys, zs
        self.field, self.component, self.amplitude = field, component, amplitude
        if len(field) == 2:
            self.field, self.component = field[0], field[1]
        self.is_first_update = True

    def _centre(self, solver):
        if self.xs is None:
            self.xs = int(solver.Nx / 2)
        if self.ys is None:
            self.ys = int(solver.Ny / 2)
        if self.zs is None:
            self.zs = int(solver.Nz / 2)

    def _write(self, solver, value):
        arr = {"E": solver.E, "H": solver.H, "J": solver.J}.get(self.field)
        if arr is None:
            return
        solver.comp(arr, "xyz".index(self.component))[self.xs, self.ys, self.zs] = value


class OracleDipole(_OraclePointSource):
    """amplitude*sin(w t + phase), f = nodes / ((zmax - zmin)/c) unless given
    (wakis/sources.py:458-565)."""

    def __init__(self, field="E", component="z", xs=None, ys=None, zs=None, nodes=10, f=None, amplitude=1.0,
                 phase=0):
        super().__init__(field, component, xs, ys, zs, amplitude)
        self.nodes, self.f, self.phase = nodes, f, phase

    def update(self, solver, t):
        if self.is_first_update:
            self._centre(solver)
            if self.f is None:
                T = (solver.z.max() - solver.z.min()) / c_light
                self.f = self.nodes / T
            self.w = 2 * np.pi * self.f
            self.is_first_update = False
        self._write(solver, self.amplitude * np.sin(self.w * t + self.phase))


class OraclePulse(_OraclePointSource):
    """Harris / Gaussian / rectangular pulse in t*c - delay of width L (default 50 dt)
    (wakis/sources.py:567-762)."""

    def __init__(self, field="E", component="z", xs=None, ys=None, zs=None, shape="Harris", L=None, amplitude=1.0,
                 delay=0.0):
        super().__init__(field, component, xs, ys, zs, amplitude)
        self.shape, self.L, self.delay = shape, L, delay
        self.tprofile = {"harris": self.harris, "gaussian": self.gaussian,
                         "rectangular": self.rectangular}[shape.lower()]

    def _harris_value(self, x):
        return (10 - 15 * np.cos(2 * np.pi / self.L * x) + 6 * np.cos(4 * np.pi / self.L * x)
                - np.cos(6 * np.pi / self.L * x)) / 32

    def harris(self, t):
        x = t * c_light - self.delay
        return self._harris_value(x) if x < self.L else 0.0

    def gaussian(self, t):
        x = t * c_light - self.delay
        return np.exp(-((x - 5 * (self.L / 10)) ** 2) / (2 * (self.L / 10) ** 2))

    def rectangular(self, t):
        x = t * c_light - self.delay
        return 1.0 if (x < self.L and x > 0.0) else 0.0

    def update(self, solver, t):
        if self.is_first_update:
            self._centre(solver)
            if self.L is None:
                self.L = 50 * solver.dt
            self.is_first_update = False
        self._write(solver, self.amplitude * self.tprofile(t))


def emsolve(solver, Nt, source=None, callback=None):
    for n in range(Nt):
        if source is not None:
            source.update(solver, n * solver.dt)
        solver.one_step()
        if solver.activate_abc:
            solver.abc_update()
        if callback is not None:
            callback(solver, n * solver.dt)


class OracleWake:
    """WakeSolver parameters and post-processing (wakis/wakeSolver.py:22-255,423-874)."""

    def __init__(self, wakelength=None, q=1e-9, sigmaz=1e-3, beta=1.0, xsource=0.0, ysource=0.0,
                 xtest=0.0, ytest=0.0, ti=None, fmax=None, skip_cells=0, counter_moving=False,
                 n_transverse_cells=1):
        # counter_moving and n_transverse_cells: wakis/wakeSolver.py:159, 190, 481-529
        self.q, self.sigmaz, self.beta = q, sigmaz, beta
        self.v = beta * c_light
        self.xsource, self.ysource, self.xtest, self.ytest = xsource, ysource, xtest, ytest
        self.fmax = self.v / (3.0 * sigmaz) if fmax is None else fmax
        self.skip_cells = skip_cells
        # injection time used by the post-processor (wakis/wakeSolver.py:166-173)
        self.ti = ti if ti is not None else 8.548921333333334 * sigmaz / (np.sqrt(beta) * self.v)
        self.wakelength = wakelength
        self.lambdas = None
        self.counter_moving = counter_moving
        self.n_transverse_cells = n_transverse_cells


def wakesolve(solver, wake, wakelength=None, compute_plane="both", record_every=None, field_monitor=None,
              j_slabs=None):
    """Runs the time loop and returns the recorded Ez slab Ezs[n] = E_z(xx, yy, :) taken
    after the beam update and before the step (wakis/routines.py:438-448); a field
    monitor is updated with E after each step (wakis/routines.py:450-451).  With a list
    j_slabs, the J_z slabs of the same lines are appended at the same point (the save_J
    dump, wakis/routines.py:444-445).  Then calls the post-processing.  Returns the
    recorded slabs (float64)."""
    if wakelength is None:
        wakelength = wake.wakelength
    ixt = np.abs(solver.x - wake.xtest).argmin()
    iyt = np.abs(solver.y - wake.ytest).argmin()
    if compute_plane.lower() == "longitudinal":
        xx, yy = ixt, iyt
    else:
        xx, yy = slice(ixt - 1, ixt + 2), slice(iyt - 1, iyt + 2)
    wake.wakelength = wakelength
    ti, v = wake.ti, wake.v
    z = solver.z
    tmax = (wakelength + ti * v + (z.max() - z.min())) / v
    Nt = int(tmax / solver.dt)
    solver.Nt = Nt
    beam = OracleBeam(q=wake.q, sigmaz=wake.sigmaz, beta=wake.beta, xsource=wake.xsource,
                      ysource=wake.ysource)
    t = np.arange(0, Nt * solver.dt, solver.dt)
    ez = solver.comp(solver.E, 2)
    slabs = []
    for n in range(Nt):
        beam.update(solver, n * solver.dt)
        slabs.append(np.array(ez[xx, yy, :], dtype=np.float64))
        if j_slabs is not None:
            j_slabs.append(np.array(solver.comp(solver.J, 2)[xx, yy, :], dtype=np.float64))
        solver.one_step()
        if field_monitor is not None:
            field_monitor.update(solver.E, solver.dt, solver.grid.shape)
    slabs = np.array(slabs)
    wake.t = t
    wake.zf = z.copy()
    wake.xf = solver.x[xx] if not isinstance(xx, (int, np.integer)) else solver.x[xx]
    wake.yf = solver.y[yy] if not isinstance(yy, (int, np.integer)) else solver.y[yy]
    wake.dz = solver.dz
    wake.Nt = Nt
    postprocess(wake, slabs, compute_plane)
    return slabs


class OracleFieldMonitor:
    """Running DFT of E (wakis/field_monitors.py:14-116): after each update the
    accumulators hold sum_n E^n * exp(-2j*pi*f*t_n), t_n = n*dt, complex128, shape
    (n_freq, Nx, Ny, Nz); dt is fixed at the first update (field_monitors.py:76-88)."""

    def __init__(self, frequencies):
        self.frequencies = np.array(frequencies)
        self.time_index = 0
        self.dt = None
        self.Ex_acc = self.Ey_acc = self.Ez_acc = None
        self.shape = None

    def update(self, E, dt, shape):
        if self.dt is None:
            self.dt = dt
            self.shape = tuple(shape)
            n = len(self.frequencies)
            self.Ex_acc = np.zeros((n, *self.shape), dtype=np.complex128)
            self.Ey_acc = np.zeros((n, *self.shape), dtype=np.complex128)
            self.Ez_acc = np.zeros((n, *self.shape), dtype=np.complex128)
        t = self.time_index * self.dt
        N = int(np.prod(self.shape))
        Ex, Ey, Ez = (comp_view(E, N, self.shape, d) for d in range(3))
        for i, f in enumerate(self.frequencies):
            phase = np.exp(-2j * np.pi * f * t)
            self.Ex_acc[i] += Ex * phase
            self.Ey_acc[i] += Ey * phase
            self.Ez_acc[i] += Ez * phase
        self.time_index += 1


def wp_index_table(wake, nt_saved, counter=False):
    """it(m, k) of the Ez(z, t) line integral (wakis/wakeSolver.py:449-529).  Evaluated
    with the reference's expression order in FP64; with counter (a counter-moving test
    charge, wakis/wakeSolver.py:500-513) loop index k reads z[-k-1] with the time
    measured from zmax.  Returns (s, it, valid, zz, nt)."""
    t = wake.t
    nt = len(t)
    dt = t[2] - t[1]
    zmin = np.min(wake.zf)
    zmax = np.max(wake.zf)
    zz = slice(wake.skip_cells, -wake.skip_cells) if wake.skip_cells != 0 else np.s_[:]
    z = wake.zf[zz]
    if wake.wakelength is None:
        wake.wakelength = nt * dt * wake.v - (zmax - zmin) - wake.ti * wake.v
    s = np.arange(-wake.ti * wake.v, wake.wakelength, dt * wake.v)
    nt = min(nt, nt_saved)
    if counter:
        ts = (z[::-1][None, :] - s[:, None]) / (-1 * wake.v) - zmax / (-1 * wake.v) - t[0] + wake.ti
    else:
        ts = (z[None, :] + s[:, None]) / wake.v - zmin / wake.v - t[0] + wake.ti
    it = np.trunc(ts / dt).astype(np.int64)
    valid = it < nt
    it = np.where(it < 0, it + nt, it)  # python negative indexing
    return s, it, valid, zz, nt


def postprocess(wake, slabs, compute_plane="both"):
    """slabs: (Nt, side, side, Nz) or (Nt, Nz).  Sets s, WP, WP_3d, WPx, WPy, f, Z, Zx,
    Zy, lambdas, lambdaf on ``wake``.  The 3-D integral reads the lines
    slab[side//2 + i, side//2 + j] for i, j in -n..n (n = n_transverse_cells, numpy
    indexing as the reference's), with the counter-moving loop when set
    (wakis/wakeSolver.py:481-529)."""
    nt_saved = slabs.shape[0]
    counter = bool(getattr(wake, "counter_moving", False)) and compute_plane.lower() != "longitudinal"
    s, it, valid, zz, nt = wp_index_table(wake, nt_saved, counter)
    dzz = np.asarray(wake.dz, dtype=np.float64)
    nz = it.shape[1]
    kk = np.broadcast_to(np.arange(nz), it.shape)
    Qn = wake.q * 1e12
    if compute_plane.lower() == "longitudinal":
        Ezt = slabs[:nt, :].T  # (Nz, nt): the 1-D branch takes the untrimmed line
        if Ezt.shape[0] != nz:
            raise ValueError("could not broadcast Ez line into the trimmed z range")
        terms = np.where(valid, Ezt[kk, np.where(valid, it, 0)] * dzz[kk], 0.0)
        WP = _seq_rows(terms) / Qn
        wake.s, wake.WP = s, WP
        calc_long_Z(wake)
        return
    n = getattr(wake, "n_transverse_cells", 1)
    c0, c1 = slabs.shape[1] // 2, slabs.shape[2] // 2
    WP = np.zeros_like(s)
    WP_3d = np.zeros((2 * n + 1, 2 * n + 1, len(s)))
    for i in range(-n, n + 1):
        for j in range(-n, n + 1):
            Ezt = slabs[:nt, c0 + i, c1 + j, zz].T  # (nz, nt)
            if counter:  # loop index k: row -k-1 of Ezt, factor -1 * dz[k]
                terms = np.where(valid, Ezt[::-1][kk, np.where(valid, it, 0)] * (-1 * dzz[kk]), 0.0)
            else:
                terms = np.where(valid, Ezt[kk, np.where(valid, it, 0)] * dzz[kk], 0.0)
            WP = _seq_rows(terms, start=WP) / Qn  # accumulator not reset (quirk)
            WP_3d[n + i, n + j, :] = WP
    wake.s, wake.WP, wake.WP_3d = s, WP_3d[n, n, :], WP_3d
    calc_trans_WP(wake)
    calc_long_Z(wake)
    calc_trans_Z(wake)


def _seq_rows(terms, start=None):
    """Sequential left-to-right sum of each row (the reference's scalar loop order)."""
    acc = np.zeros(terms.shape[0]) if start is None else start.copy()
    for k in range(terms.shape[1]):
        acc = acc + terms[:, k]
    return acc


def calc_trans_WP(wake):
    """Panofsky-Wenzel transverse wake (wakis/wakeSolver.py:553-626)."""
    s = wake.s
    ds = s[2] - s[1]
    ns = len(s)
    c = getattr(wake, "n_transverse_cells", 1)
    int_WP = np.zeros_like(wake.WP_3d)
    for n in range(ns):
        int_WP[:, :, n] = np.sum(wake.WP_3d[:, :, 0:n], axis=2) * ds
    dxf, dyf = np.diff(wake.xf), np.diff(wake.yf)
    wake.WPx = -(int_WP[c + 1, c, :] - int_WP[c - 1, c, :]) / (dxf[c - 1] + dxf[c])
    wake.WPy = -(int_WP[c, c + 1, :] - int_WP[c, c - 1, :]) / (dyf[c - 1] + dyf[c])


def calc_lambdas_analytic(wake):
    """wakis/wakeSolver.py:842-874."""
    wake.lambdas = 1 / (wake.sigmaz * np.sqrt(2 * np.pi)) * np.exp(-(wake.s ** 2) / (2 * wake.sigmaz ** 2))


def dft_setup(wake, samples=1001, fmax=None):
    ds = np.mean(wake.s[1:] - wake.s[:-1])
    fmax = wake.fmax if fmax is None else fmax
    N = int((wake.v / ds) // fmax * samples)
    ffft = np.fft.fftfreq(N, ds / wake.v)
    mask = np.logical_and(ffft >= 0, ffft < fmax)
    return ds, N, ffft, mask


def calc_long_Z(wake, samples=1001, fmax=None):
    """wakis/wakeSolver.py:628-720."""
    if wake.lambdas is None:
        calc_lambdas_analytic(wake)
    ds, N, ffft, mask = dft_setup(wake, samples, fmax)
    lambdafft = np.fft.fft(wake.lambdas * wake.v, n=N)
    WPfft = np.fft.fft(wake.WP * 1e12, n=N)
    WPf = WPfft[mask] * ds
    lambdaf = lambdafft[mask] * ds
    wake.f = ffft[mask]
    wake.Z = -WPf / lambdaf
    wake.lambdaf = lambdaf


def calc_trans_Z(wake, samples=1001, fmax=None):
    """wakis/wakeSolver.py:722-785."""
    ds, N, ffft, mask = dft_setup(wake, samples, fmax)
    lambdafft = np.fft.fft(wake.lambdas * wake.v, n=N)
    lambdaf = lambdafft[mask] * ds
    wake.Zx = 1j * (np.fft.fft(wake.WPx * 1e12, n=N)[mask] * ds) / lambdaf
    wake.Zy = 1j * (np.fft.fft(wake.WPy * 1e12, n=N)[mask] * ds) / lambdaf
