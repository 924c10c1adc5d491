"""Parity cases shared by the fixture generator (make_golden.py), the oracle pins and
the GPU parity tests.

Each case is a small, seeded configuration that exercises one part of the FIT path:
the wake run with the 3x3 Ez line integral, lossy walls with the relaxation-time
conductivity and z PML, plane-wave / wave-packet hard sources, the analytic
resonator, mixed PEC/PMC/periodic/ABC/PML faces on a non-uniform grid (row-crossing
neighbours live), and FP32 vs FP64 storage.  Geometry is analytic: masks are
evaluated at cell centres (or at cell corners for the test_001 "legacy" rule).
"""

import numpy as np

MM = 1e-3


# ----------------------------------------------------------------------------- masks
def cube_pipe(X, Y, Z, half=25 * MM, r=5 * MM):
    """Vacuum region of the cavity configs: a cube union a cylindrical pipe along z."""
    return ((np.abs(X) <= half) & (np.abs(Y) <= half) & (np.abs(Z) <= half)) | (X ** 2 + Y ** 2 <= r ** 2)


def walls(X, Y, Z, half=25 * MM, r=5 * MM):
    return ~cube_pipe(X, Y, Z, half, r)


def sphere(X, Y, Z, R=0.25):
    return X ** 2 + Y ** 2 + Z ** 2 <= R ** 2


def block(X, Y, Z, lo, hi):
    return ((X >= lo[0]) & (X <= hi[0]) & (Y >= lo[1]) & (Y <= hi[1]) & (Z >= lo[2]) & (Z <= hi[2]))


def test001_boxes_corner_rule(x, y, z, tol):
    """Cell mask of the test_001 cubic cavity: union of |x|,|y|<=25mm & |z|<=15mm and
    |x|,|y|<=7.5mm & |z|<=50mm; a cell is inside when any of its 8 corners is inside
    (the reference's default 'legacy' STL rule)."""
    X, Y, Z = np.meshgrid(x, y, z, indexing="ij")
    inside = (((np.abs(X) <= 25 * MM + tol) & (np.abs(Y) <= 25 * MM + tol) & (np.abs(Z) <= 15 * MM + tol))
              | ((np.abs(X) <= 7.5 * MM + tol) & (np.abs(Y) <= 7.5 * MM + tol) & (np.abs(Z) <= 50 * MM + tol)))
    m = np.zeros((len(x) - 1, len(y) - 1, len(z) - 1), dtype=bool)
    for a in (0, 1):
        for b in (0, 1):
            for c in (0, 1):
                m |= inside[a:a + m.shape[0], b:b + m.shape[1], c:c + m.shape[2]]
    return m


def centres(x, y, z):
    xc = x[:-1] + np.diff(x) / 2
    yc = y[:-1] + np.diff(y) / 2
    zc = z[:-1] + np.diff(z) / 2
    return np.meshgrid(xc, yc, zc, indexing="ij")


def nonuniform_axis(lo, hi, n, seed):
    rng = np.random.default_rng(seed)
    w = rng.uniform(0.6, 1.4, n)
    e = np.concatenate([[0.0], np.cumsum(w)])
    return lo + (hi - lo) * e / e[-1]


# ----------------------------------------------------------------------------- cases
def _axes(c):
    g = c["grid"]
    if "x" in g:
        return np.asarray(g["x"]), np.asarray(g["y"]), np.asarray(g["z"])
    return (np.linspace(g["xmin"], g["xmax"], g["Nx"] + 1), np.linspace(g["ymin"], g["ymax"], g["Ny"] + 1),
            np.linspace(g["zmin"], g["zmax"], g["Nz"] + 1))


def solids_for(c):
    """[(name, mask (Nx,Ny,Nz) bool, material list)] of a case."""
    x, y, z = _axes(c)
    X, Y, Z = centres(x, y, z)
    out = []
    for name, kind, params, mat in c.get("solids", []):
        if kind == "cube_pipe":
            m = cube_pipe(X, Y, Z, **params)
        elif kind == "walls":
            m = walls(X, Y, Z, **params)
        elif kind == "sphere":
            m = sphere(X, Y, Z, **params)
        elif kind == "block":
            m = block(X, Y, Z, **params)
        else:
            raise KeyError(kind)
        out.append((name, m, list(mat)))
    return out


_cavity_grid = dict(xmin=-30 * MM, xmax=30 * MM, ymin=-30 * MM, ymax=30 * MM, zmin=-60 * MM, zmax=60 * MM)

CASES = {
    # the 60x60x120 cavity geometry at reduced size: PEC background, vacuum cube + pipe, ABC in z
    "cavity_f64": dict(
        kind="wake", dtype="float64", grid=dict(_cavity_grid, Nx=16, Ny=16, Nz=32),
        solids=[("cavity", "cube_pipe", {}, [1.0, 1.0])], bg="pec",
        bc_low=["pec", "pec", "abc"], bc_high=["pec", "pec", "abc"], cfln=1.0,
        wake=dict(q=1e-9, sigmaz=10 * MM, beta=1.0, xsource=0.0, ysource=0.0, xtest=0.0, ytest=0.0,
                  fmax=5e9, skip_cells=0),
        wakelength=0.1, compute_plane="both"),
    # the cavity wake with a counter-moving test charge (3-D integral down z from zmax) and
    # skip_cells (dz indexed by the loop index)
    "counter_f64": dict(
        kind="wake", dtype="float64", grid=dict(_cavity_grid, Nx=16, Ny=16, Nz=32),
        solids=[("cavity", "cube_pipe", {}, [1.0, 1.0])], bg="pec",
        bc_low=["pec", "pec", "abc"], bc_high=["pec", "pec", "abc"], cfln=1.0,
        wake=dict(q=1e-9, sigmaz=10 * MM, beta=1.0, xsource=0.0, ysource=0.0, xtest=0.0, ytest=0.0,
                  fmax=5e9, skip_cells=2, counter_moving=True),
        wakelength=0.1, compute_plane="both"),
    # the lossy 128x128x256 cavity physics at reduced size: sigma=1e4 walls (relaxation form), z PML, beta 0.8, offset 2 mm.
    # CFL 0.5 (the reference default): with sigma>0 cells the reference's explicit loss term
    # diverges at CFL 1.0 on this grid.
    "lossy_f64": dict(
        kind="wake", dtype="float64", grid=dict(_cavity_grid, Nx=16, Ny=16, Nz=40),
        solids=[("walls", "walls", {}, [1.0, 1.0, 1e4])], bg=[1.0, 1.0],
        bc_low=["pec", "pec", "pml"], bc_high=["pec", "pec", "pml"], n_pml=4, cfln=0.5,
        wake=dict(q=1e-9, sigmaz=10 * MM, beta=0.8, xsource=2 * MM, ysource=0.0, xtest=2 * MM, ytest=0.0,
                  fmax=5e9, skip_cells=0),
        wakelength=0.05, compute_plane="both"),
    "lossy_f32": dict(
        kind="wake", dtype="float32", grid=dict(_cavity_grid, Nx=16, Ny=16, Nz=40),
        solids=[("walls", "walls", {}, [1.0, 1.0, 1e4])], bg=[1.0, 1.0],
        bc_low=["pec", "pec", "pml"], bc_high=["pec", "pec", "pml"], n_pml=4, cfln=0.5,
        wake=dict(q=1e-9, sigmaz=10 * MM, beta=0.8, xsource=2 * MM, ysource=0.0, xtest=2 * MM, ytest=0.0,
                  fmax=5e9, skip_cells=0),
        wakelength=0.05, compute_plane="both"),
    # longitudinal-only post-processing on a non-uniform z axis
    "longitudinal_f64": dict(
        kind="wake", dtype="float64",
        grid=dict(x=np.linspace(-30 * MM, 30 * MM, 15), y=np.linspace(-30 * MM, 30 * MM, 15),
                  z=nonuniform_axis(-60 * MM, 60 * MM, 30, seed=11)),
        solids=[("cavity", "cube_pipe", {}, [1.0, 1.0])], bg="pec",
        bc_low=["pec", "pec", "pec"], bc_high=["pec", "pec", "pec"], cfln=0.9,
        wake=dict(q=1e-9, sigmaz=12 * MM, beta=1.0, xsource=0.0, ysource=0.0, xtest=0.0, ytest=0.0,
                  fmax=4e9, skip_cells=0),
        wakelength=0.08, compute_plane="longitudinal"),
    # skip_cells on a non-uniform z axis (dz indexed untrimmed)
    "skip_nonuniform_f64": dict(
        kind="wake", dtype="float64",
        grid=dict(x=np.linspace(-30 * MM, 30 * MM, 13), y=np.linspace(-30 * MM, 30 * MM, 14),
                  z=nonuniform_axis(-60 * MM, 60 * MM, 28, seed=12)),
        solids=[("cavity", "cube_pipe", {}, [1.0, 1.0])], bg="pec",
        bc_low=["pec", "pec", "pec"], bc_high=["pec", "pec", "pec"], cfln=1.0,
        wake=dict(q=1e-9, sigmaz=12 * MM, beta=1.0, xsource=1 * MM, ysource=-1 * MM, xtest=0.0, ytest=0.0,
                  fmax=4e9, skip_cells=3),
        wakelength=0.08, compute_plane="both"),
    # test_005 layout: periodic x/y, PEC z-lo, PML z-hi, plane wave, dt overridden by a Python float
    "planewave_f32": dict(
        kind="emsolve", dtype="float32",
        grid=dict(xmin=-1.0, xmax=1.0, ymin=-1.0, ymax=1.0, zmin=0.0, zmax=1.0, Nx=6, Ny=6, Nz=60),
        solids=[], bg=[1.0, 1.0, 0.0], bc_low=["periodic", "periodic", "pec"],
        bc_high=["periodic", "periodic", "pml"], n_pml=10, cfln=0.5,
        source=dict(type="PlaneWave", xs=(0, 6), ys=(0, 6), zs=0, beta=1.0, amplitude=100.0,
                    f_nodes=15, nodes=7, phase=np.pi / 2),
        dt_override="1/f/200", Nt=150),
    # test_003 layout at reduced size: plane wave (f = 15 nodes over the domain, source on
    # the interior cells of plane 1, default dt) onto a dielectric sphere eps_r = 10,
    # periodic x/y, PEC z-lo, PML z-hi
    "planewave_sphere_f32": dict(
        kind="emsolve", dtype="float32",
        grid=dict(xmin=-6 * MM, xmax=6 * MM, ymin=-6 * MM, ymax=6 * MM, zmin=-15 * MM, zmax=15 * MM,
                  Nx=12, Ny=12, Nz=24),
        solids=[("Sphere", "sphere", {"R": 5 * MM}, [10.0, 1.0])], bg=[1.0, 1.0],
        bc_low=["periodic", "periodic", "pec"], bc_high=["periodic", "periodic", "pml"], n_pml=10, cfln=0.5,
        source=dict(type="PlaneWave", xs=(1, 11), ys=(1, 11), zs=1, beta=1.0, amplitude=1.0,
                    f_nodes=15, nodes=None, phase=0),
        Nt=90),
    # the 256^3 sphere layout at reduced size: PML on all faces, dielectric sphere, wave packet
    "wavepacket_f64": dict(
        kind="emsolve", dtype="float64",
        grid=dict(xmin=-1.0, xmax=1.0, ymin=-1.0, ymax=1.0, zmin=-1.0, zmax=1.0, Nx=16, Ny=16, Nz=16),
        solids=[("sphere", "sphere", {"R": 0.25}, [2.0, 1.0])], bg=[1.0, 1.0],
        bc_low=["pml", "pml", "pml"], bc_high=["pml", "pml", "pml"], n_pml=3, cfln=0.5,
        source=dict(type="WavePacket", zs=4, sigmaz=0.3, sigmaxy=10.0, wavelength=0.5, amplitude=1.0),
        Nt=60, probes=8),
    # test_002 layout: TE101 mode of a PEC cube, H initialised analytically
    "resonator_f64": dict(kind="resonator", dtype="float64", N=10, Nt=120),
    # odd sizes, non-uniform axes, PMC/PEC/periodic/ABC/PML faces, dielectric + lossy blocks,
    # random initial fields, emsolve with the ABC update (row-crossing neighbours live)
    "mixed_bc_f64": dict(
        kind="emsolve", dtype="float64",
        grid=dict(x=nonuniform_axis(-1.0, 1.0, 10, seed=21), y=nonuniform_axis(-1.0, 1.0, 9, seed=22),
                  z=nonuniform_axis(-1.0, 1.0, 12, seed=23)),
        solids=[("diel", "block", {"lo": (-0.5, -0.5, -0.2), "hi": (0.3, 0.4, 0.5)}, [4.0, 2.0]),
                ("lossy", "block", {"lo": (0.2, -1.0, -1.0), "hi": (1.0, 0.0, 0.0)}, [1.0, 1.0, 50.0])],
        bg=[1.0, 1.0], bc_low=["pmc", "periodic", "abc"], bc_high=["pec", "periodic", "pml"], n_pml=3,
        cfln=0.7, random_init=31, Nt=15),
    # PMC faces ('magnetic' and 'pmc'), lossy block, user loop of beam.update + one_step
    "pmc_beam_f64": dict(
        kind="userloop", dtype="float64", grid=dict(_cavity_grid, Nx=12, Ny=10, Nz=24),
        solids=[("lossy", "block", {"lo": (-0.03, -0.03, 0.02), "hi": (0.03, 0.03, 0.06)}, [3.0, 1.0, 20.0])],
        bg=[1.0, 1.0], bc_low=["magnetic", "pec", "pec"], bc_high=["pmc", "pec", "pec"], cfln=0.8,
        beam=dict(q=1e-9, sigmaz=10 * MM, beta=1.0, xsource=0.0, ysource=0.0), Nt=40),
    # periodic x and y with a conductive background: live row-crossing couplings, FP32
    "periodic_cond_f32": dict(
        kind="emsolve", dtype="float32",
        grid=dict(xmin=-1.0, xmax=1.0, ymin=-1.0, ymax=1.0, zmin=-1.0, zmax=1.0, Nx=8, Ny=6, Nz=10),
        solids=[], bg=[2.0, 1.0, 0.5], bc_low=["periodic", "periodic", "pec"],
        bc_high=["periodic", "periodic", "pec"], cfln=0.5, random_init=41, Nt=20),
}

# point / region hard sources driven through the Field API every step (emsolve host loop)
_box = dict(xmin=-1.0, xmax=1.0, ymin=-1.0, ymax=1.0, zmin=-1.0, zmax=1.0)
CASES["dipole_f64"] = dict(
    kind="emsolve", dtype="float64", grid=dict(_box, Nx=12, Ny=12, Nz=16),
    solids=[("diel", "block", {"lo": (-0.6, -0.6, 0.2), "hi": (0.5, 0.4, 0.8)}, [3.0, 1.0])], bg=[1.0, 1.0],
    bc_low=["pec", "pec", "pec"], bc_high=["pec", "pec", "pec"], cfln=0.5, Nt=120,
    source=dict(type="Dipole", field="E", component="z", nodes=3, amplitude=2.0, phase=0.4))
CASES["pulse_harris_f32"] = dict(
    kind="emsolve", dtype="float32", grid=dict(_box, Nx=14, Ny=12, Nz=18),
    solids=[("lossy", "block", {"lo": (-1.0, -1.0, 0.3), "hi": (1.0, 1.0, 0.7)}, [1.0, 1.0, 20.0])],
    bg=[1.0, 1.0], bc_low=["pec", "pec", "pml"], bc_high=["pec", "pec", "pml"], n_pml=3, cfln=0.5, Nt=140,
    source=dict(type="Pulse", field="Hy", shape="Harris", xs=(4, 9), ys=6, zs=5, L=0.8, amplitude=1.5))
CASES["pulse_gauss_j_f64"] = dict(
    kind="emsolve", dtype="float64", grid=dict(_box, Nx=10, Ny=12, Nz=14),
    solids=[("lossy", "block", {"lo": (-0.4, -0.4, -0.4), "hi": (0.4, 0.4, 0.4)}, [2.0, 1.0, 5.0])],
    bg=[1.0, 1.0], bc_low=["pec", "pml", "pec"], bc_high=["pec", "pml", "pec"], n_pml=3, cfln=0.5, Nt=100,
    source=dict(type="Pulse", field="J", component="x", shape="Gaussian", xs=5, ys=6, zs=7, L=1.0, amplitude=1e3))
CASES["pulse_rect_f64"] = dict(
    kind="emsolve", dtype="float64", grid=dict(_box, Nx=12, Ny=10, Nz=12),
    solids=[], bg=[1.0, 1.0], bc_low=["pec", "pec", "pec"], bc_high=["pec", "pec", "pec"], cfln=0.5, Nt=90,
    source=dict(type="Pulse", field="Ex", shape="Rectangular", xs=(3, 8), ys=(2, 5), zs=6, L=0.6,
                delay=0.05, amplitude=0.7))


def point_source(module, sc):
    """A Dipole or Pulse of `module.sources` from a case's source description (index
    spans given as (start, stop) become slices)."""
    kw = {k: (slice(*v) if k in ("xs", "ys", "zs") and isinstance(v, tuple) else v)
          for k, v in sc.items() if k != "type"}
    return getattr(module.sources, sc["type"])(**kw)


# wake runs with a FieldMonitor (running DFT of E after every step) attached
CASES["monitor_f64"] = dict(CASES["cavity_f64"], monitor=[1.0e9, 3.0e9, 4.5e9])
CASES["monitor_f32"] = dict(CASES["lossy_f32"], monitor=[2.0e9, 5.0e9])


def axes(c):
    return _axes(c)


def random_fields(N, seed, dtype):
    rng = np.random.default_rng(seed)
    return rng.standard_normal(3 * N).astype(dtype), rng.standard_normal(3 * N).astype(dtype)


def probe_points(c):
    """Seeded interior probe cells (outside the PML) for the emsolve cases."""
    x, y, z = axes(c)
    n = c.get("probe_margin", c.get("n_pml", 0))
    rng = np.random.default_rng(2)
    Nx, Ny, Nz = len(x) - 1, len(y) - 1, len(z) - 1
    return np.stack([rng.integers(n, Nx - n, c["probes"]), rng.integers(n, Ny - n, c["probes"]),
                     rng.integers(n, Nz - n, c["probes"])], axis=1)


def resonator_H(N, dt):
    """Analytic TE101 H field at t=-dt/2 on the test_002 grid, written as the reference's
    test does (cell index ii -> x = ii*dx + xmin)."""
    from scipy.constants import c as c_light
    L = 1.0
    d = L / N
    xmin = -L / 2 + d / 2
    ii = np.arange(N)
    x = ii * d + xmin
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    t = -0.5 * dt
    m, n, p = 1, 0, 1
    h2 = (m * np.pi / L) ** 2 + (n * np.pi / L) ** 2 + (p * np.pi / L) ** 2
    ct = np.cos(np.sqrt(2) * np.pi / L * c_light * t)
    Hz = np.cos(m * np.pi / L * (X - L / 2)) * np.cos(n * np.pi / L * (Y - L / 2)) * np.sin(p * np.pi / L * (Z - L / 2)) * ct
    Hy = (-2 / h2 * (n * np.pi / L) * (p * np.pi / L) * np.cos(m * np.pi / L * (X - L / 2))
          * np.sin(n * np.pi / L * (Y - L / 2)) * np.cos(p * np.pi / L * (Z - L / 2)) * ct)
    Hx = (-2 / h2 * (m * np.pi / L) * (p * np.pi / L) * np.sin(m * np.pi / L * (X - L / 2))
          * np.cos(n * np.pi / L * (Y - L / 2)) * np.cos(p * np.pi / L * (Z - L / 2)) * ct)
    return Hx, Hy, Hz, (xmin, xmin + L)


# ----------------------------------------------------------------------------- checkpoints
# save_state after save_at steps of a user loop, a fresh solver load_state + the remaining
# steps, and the uninterrupted run (wakis/solverFIT3D.py:908-1035); emsolve(save=True)
# (wakis/routines.py:122-204) on a small PEC box.
CHECKPOINT_CASES = {
    "checkpoint_pmc_beam_f64": dict(base="pmc_beam_f64", save_at=17),
}
EMSOLVE_SAVE_CASE = dict(grid=dict(xmin=-1.0, xmax=1.0, ymin=-1.0, ymax=1.0, zmin=-1.0, zmax=1.0, Nx=8, Ny=8, Nz=8),
                         Nt=4, fields=["E", "Hy"], components=["Abs", "z"])


# ----------------------------------------------------------------------------- mesh refinement
# GridFIT3D.refine_axis (wakis/gridFIT3D.py:771-859) on seeded snap sets: (seed, xmin, xmax,
# nodes, number of snaps, method)
REFINE_CASES = [(31, -0.06, 0.06, 31, 4, "insert"), (32, -0.06, 0.06, 31, 4, "neighbor"),
                (33, 0.0, 1.0, 25, 6, "insert"), (34, -1.0, 2.0, 41, 3, "neighbor"),
                (35, -0.2, 0.2, 17, 2, "insert"), (36, 0.0, 0.5, 60, 9, "neighbor")]


def refine_snaps(seed, xmin, xmax, nsnap):
    """Snap coordinates of a refinement case: the domain bounds and nsnap interior points."""
    rng = np.random.default_rng(seed)
    inner = np.sort(rng.uniform(xmin + 0.05 * (xmax - xmin), xmax - 0.05 * (xmax - xmin), nsnap))
    return np.unique(np.concatenate(([xmin], np.round(inner, 5), [xmax])))


# ----------------------------------------------------------------------------- full configs
# The benchmark workloads at full size (geometry analytic, evaluated at cell centres).
WORKLOADS = {
    # plain FP64 PEC cubic cavity, 60x60x120, ABC in z, CFL 1.0, wake 0.5 m, fmax 5 GHz
    "cavity_60x60x120": dict(
        kind="wake", dtype="float64", grid=dict(_cavity_grid, Nx=60, Ny=60, Nz=120),
        solids=[("cavity", "cube_pipe", {}, [1.0, 1.0])], bg="pec",
        bc_low=["pec", "pec", "abc"], bc_high=["pec", "pec", "abc"], cfln=1.0,
        wake=dict(q=1e-9, sigmaz=10 * MM, beta=1.0, xsource=0.0, ysource=0.0, xtest=0.0, ytest=0.0,
                  fmax=5e9, skip_cells=0),
        wakelength=0.5, compute_plane="both"),
    # lossy cavity, run a: 128x128x256, sigma = 1e4 walls (relaxation form), 10-cell z PML, beta 1
    # (CFL 0.5: the reference's explicit loss term diverges at CFL 1.0 with sigma > 0 cells)
    "lossy_cavity_128x128x256": dict(
        kind="wake", dtype="float32", grid=dict(_cavity_grid, Nx=128, Ny=128, Nz=256),
        solids=[("walls", "walls", {}, [1.0, 1.0, 1e4])], bg=[1.0, 1.0],
        bc_low=["pec", "pec", "pml"], bc_high=["pec", "pec", "pml"], n_pml=10, cfln=0.5,
        wake=dict(q=1e-9, sigmaz=10 * MM, beta=1.0, xsource=0.0, ysource=0.0, xtest=0.0, ytest=0.0,
                  fmax=5e9, skip_cells=0),
        wakelength=1.0, compute_plane="both"),
    # lossy cavity, run b: beta 0.8, source and test offset 2 mm in x
    "lossy_cavity_128x128x256_offset": dict(
        kind="wake", dtype="float32", grid=dict(_cavity_grid, Nx=128, Ny=128, Nz=256),
        solids=[("walls", "walls", {}, [1.0, 1.0, 1e4])], bg=[1.0, 1.0],
        bc_low=["pec", "pec", "pml"], bc_high=["pec", "pec", "pml"], n_pml=10, cfln=0.5,
        wake=dict(q=1e-9, sigmaz=10 * MM, beta=0.8, xsource=2 * MM, ysource=0.0, xtest=2 * MM, ytest=0.0,
                  fmax=5e9, skip_cells=0),
        wakelength=1.0, compute_plane="both"),
    # sphere and wave packet: unit box [-1,1]^3 on 256^3, 12-cell PML on all faces, sphere r=0.25 eps_r=2,
    # x-polarised wave packet along +z, centre wavelength 0.2, 2000 steps, 64 probes
    "sphere_packet_256": dict(
        kind="emsolve", dtype="float32",
        grid=dict(xmin=-1.0, xmax=1.0, ymin=-1.0, ymax=1.0, zmin=-1.0, zmax=1.0, Nx=256, Ny=256, Nz=256),
        solids=[("sphere", "sphere", {"R": 0.25}, [2.0, 1.0])], bg=[1.0, 1.0],
        bc_low=["pml", "pml", "pml"], bc_high=["pml", "pml", "pml"], n_pml=12, cfln=0.5,
        source=dict(type="WavePacket", zs=13, sigmaz=0.3, sigmaxy=100.0, wavelength=0.2, amplitude=1.0),
        Nt=2000, probes=64),
}


# ----------------------------------------------------------------------------- Ez files
# WakeSolver post-processing of a recorded Ez line history (no solver run): seeded
# synthetic histories with the reference's Ez.h5 keys, non-uniform dz, FP32-valued slabs.
WAKE_FILE_CASES = {
    "wakefile_3d": dict(seed=21, nz=40, nt=320, t0=0.0, shape3=True, plane="both",
                        wake=dict(q=1e-9, sigmaz=2e-3, wakelength=0.02, beta=1.0, skip_cells=0)),
    # skip_cells trims z; t0 > 0 makes early taps' time index negative (wraps in the reference)
    "wakefile_3d_skip_t0": dict(seed=22, nz=40, nt=320, t0=12e-12, shape3=True, plane="both",
                                wake=dict(q=1e-9, sigmaz=2e-3, wakelength=0.02, beta=1.0, skip_cells=2)),
    # beta 0.8, a history too short for the late taps, longitudinal from 1-D slabs
    "wakefile_long_1d": dict(seed=23, nz=40, nt=200, t0=0.0, shape3=False, plane="longitudinal",
                             wake=dict(q=1e-9, sigmaz=2e-3, wakelength=0.02, beta=0.8, skip_cells=0)),
    # a counter-moving test charge (the 3-D integral runs down z from zmax with -dz),
    # with skip_cells, and with t0 > 0 (wrapped negative time indices)
    "wakefile_3d_counter": dict(seed=24, nz=40, nt=320, t0=0.0, shape3=True, plane="both",
                                wake=dict(q=1e-9, sigmaz=2e-3, wakelength=0.02, beta=1.0, skip_cells=2,
                                          counter_moving=True)),
    "wakefile_3d_counter_t0": dict(seed=25, nz=40, nt=320, t0=12e-12, shape3=True, plane="both",
                                   wake=dict(q=1e-9, sigmaz=2e-3, wakelength=0.02, beta=0.9, skip_cells=0,
                                             counter_moving=True)),
    # 5x5 slabs integrated over n_transverse_cells = 2 (25 lines)
    "wakefile_5x5_n2": dict(seed=26, nz=40, nt=320, t0=0.0, shape3=True, side=5, n_transverse_cells=2,
                            plane="both", wake=dict(q=1e-9, sigmaz=2e-3, wakelength=0.02, beta=1.0, skip_cells=1)),
}


def synthetic_history(seed, nz=40, nt=320, shape3=True, t0=0.0, side=3):
    """(meta, slabs): meta holds the x, y, z, dx, dy, dz, t datasets of an Ez file; slabs
    (nt, side, side, nz) or (nt, nz) float64 holding FP32 values."""
    rng = np.random.default_rng(seed)
    dz = 1e-3 * (0.8 + 0.4 * rng.random(nz))
    zedges = np.concatenate([[-0.02], -0.02 + np.cumsum(dz)])
    z = 0.5 * (zedges[1:] + zedges[:-1])
    dt = 0.45 * dz.min() / 299792458.0
    t = t0 + np.arange(0, nt * dt, dt)[:nt]
    if side == 3:
        x = np.array([-1.1e-3, 0.0, 0.9e-3])
        y = np.array([-0.8e-3, 0.0, 1.2e-3])
    else:
        x = np.linspace(-1.0e-3, 1.1e-3, side) ** 3 * 1e6
        y = np.linspace(-1.2e-3, 0.9e-3, side) ** 3 * 1e6
    shape = (nt, side, side, nz) if shape3 else (nt, nz)
    slabs = rng.standard_normal(shape).astype(np.float32).astype(np.float64) * 1e3
    return dict(x=x, y=y, z=z, dx=np.full(side, 1e-3), dy=np.full(side, 1e-3), dz=dz, t=t), slabs
