"""Generate the golden fixtures under tests/golden/ by running the REFERENCE Wakis code.

Run from the repository root in a container that holds the reference checkout:

    python tests/golden/make_golden.py /path/to/reference            # all small cases
    python tests/golden/make_golden.py /path/to/reference --test001  # + the test_001 run (~2 min)

The reference imports h5py, pyvista and matplotlib, which are absent here; the
test-only stand-ins in tests/golden/_standins/ replace them (in-memory HDF5, a dict
StructuredGrid, an empty pyplot).  STL voxelisation needs VTK, so solid masks are
injected analytically into ``grid.grid[key]`` (C order over (Nx, Ny, Nz), which is how
``SolverFIT3D._apply_stl_materials`` reshapes them).  Fixtures are written as .npz.
This script is the only place that executes reference code; nothing at test time
reads the reference checkout.
"""

import argparse
import os
import re
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import cases as C  # noqa: E402


def load_reference(ref_root):
    sys.path.insert(0, os.path.join(HERE, "_standins"))
    sys.path.insert(0, ref_root)
    import wakis  # noqa: F401
    return wakis


def make_grid(wakis, case):
    x, y, z = C.axes(case)
    g = case["grid"]
    if "x" in g:
        grid = wakis.GridFIT3D(x=x, y=y, z=z, verbose=0)
    else:
        grid = wakis.GridFIT3D(g["xmin"], g["xmax"], g["ymin"], g["ymax"], g["zmin"], g["zmax"],
                               g["Nx"], g["Ny"], g["Nz"], verbose=0)
    solids = C.solids_for(case)
    if solids:
        grid.stl_solids = {n: n + ".stl" for n, _, _ in solids}
        grid.stl_materials = {n: mat for n, _, mat in solids}
        grid.stl_colors = {n: "white" for n, _, _ in solids}
        for n, m, _ in solids:
            grid.grid[n] = m.reshape(-1)  # C order, as the solver reshapes it
    return grid


def make_solver(wakis, case, grid, wake=None):
    dtype = np.float32 if case["dtype"] == "float32" else np.float64
    return wakis.SolverFIT3D(grid, wake, cfln=case.get("cfln", 0.5), bc_low=list(case["bc_low"]),
                             bc_high=list(case["bc_high"]), use_stl=bool(case.get("solids")),
                             bg=case["bg"], dtype=dtype, n_pml=case.get("n_pml", 10), verbose=0)


def run_wake(wakis, name, case, out):
    w = case["wake"]
    grid = make_grid(wakis, case)
    wake = wakis.WakeSolver(wakelength=case["wakelength"], save=False, verbose=0,
                            Ez_file=os.path.join(os.getcwd(), name + "_Ez.h5"), **w)
    solver = make_solver(wakis, case, grid, wake)
    mon = None
    kw = {}
    if "monitor" in case:
        from wakis.field_monitors import FieldMonitor
        mon = FieldMonitor(case["monitor"])
        kw = dict(use_field_monitor=True, field_monitor=mon)
    solver.wakesolve(wakelength=case["wakelength"], compute_plane=case["compute_plane"], **kw)
    res = dict(Nt=solver.Nt, dt=np.float64(solver.dt), s=wake.s, WP=wake.WP, f=wake.f, Z=wake.Z,
               lambdas=wake.lambdas, E=solver.E.toarray(), H=solver.H.toarray(), J=solver.J.toarray())
    if mon is not None:
        comps = mon.get_components()
        res.update(Ex_acc=comps["Ex"], Ey_acc=comps["Ey"], Ez_acc=comps["Ez"])
    if case["compute_plane"] != "longitudinal":
        res.update(WP_3d=wake.WP_3d, WPx=wake.WPx, WPy=wake.WPy, Zx=wake.Zx, Zy=wake.Zy)
    out[name] = res


def run_emsolve(wakis, name, case, out):
    from scipy.constants import c as c_light
    grid = make_grid(wakis, case)
    solver = make_solver(wakis, case, grid)
    src = None
    sc = case.get("source")
    if sc is not None and sc["type"] == "PlaneWave":
        f = sc["f_nodes"] / ((solver.z.max() - solver.z.min()) / c_light)
        src = wakis.sources.PlaneWave(xs=slice(*sc["xs"]), ys=slice(*sc["ys"]), zs=sc["zs"], beta=sc["beta"],
                                      amplitude=sc["amplitude"], f=f, nodes=sc["nodes"], phase=sc["phase"])
        if case.get("dt_override") == "1/f/200":
            solver.dt = 1 / f / 200
    elif sc is not None and sc["type"] == "WavePacket":
        src = wakis.sources.WavePacket(zs=sc["zs"], sigmaz=sc["sigmaz"], sigmaxy=sc["sigmaxy"],
                                       wavelength=sc["wavelength"], amplitude=sc["amplitude"])
    elif sc is not None:
        src = C.point_source(wakis, sc)
    if "random_init" in case:
        E0, H0 = C.random_fields(solver.N, case["random_init"], solver.E.toarray().dtype)
        solver.E.fromarray(E0)
        solver.H.fromarray(H0)
    probes = []
    if "probes" in case:
        P = C.probe_points(case)

        def cb(s, t):
            probes.append([s.E[int(i), int(j), int(k), "z"] for i, j, k in P])
    else:
        cb = None
    solver.emsolve(case["Nt"], source=src, callback=cb)
    res = dict(dt=np.float64(solver.dt), E=solver.E.toarray(), H=solver.H.toarray(), J=solver.J.toarray())
    if probes:
        res["probes"] = np.array(probes, dtype=np.float64)
    out[name] = res


def run_resonator(wakis, name, case, out):
    N = case["N"]
    d = 1.0 / N
    grid = wakis.GridFIT3D(-0.5 + d / 2, 0.5 + d / 2, -0.5 + d / 2, 0.5 + d / 2, -0.5 + d / 2, 0.5 + d / 2,
                           N, N, N, verbose=0)
    solver = wakis.SolverFIT3D(grid, bc_low=["pec"] * 3, bc_high=["pec"] * 3, verbose=0)
    Hx, Hy, Hz, _ = C.resonator_H(N, solver.dt)
    solver.H[:, :, :, "x"] = Hx
    solver.H[:, :, :, "y"] = Hy
    solver.H[:, :, :, "z"] = Hz
    ey = []
    for _ in range(case["Nt"]):
        ey.append(solver.E[N // 2, N // 2, N // 2, "y"])
        solver.one_step()
    out[name] = dict(dt=np.float64(solver.dt), Ey=np.array(ey), E=solver.E.toarray(), H=solver.H.toarray())


def run_userloop(wakis, name, case, out):
    grid = make_grid(wakis, case)
    solver = make_solver(wakis, case, grid)
    beam = wakis.sources.Beam(**case["beam"])
    for n in range(case["Nt"]):
        beam.update(solver, n * solver.dt)
        solver.one_step()
    out[name] = dict(dt=np.float64(solver.dt), E=solver.E.toarray(), H=solver.H.toarray(), J=solver.J.toarray())


def run_checkpoint(wakis, name, spec, out):
    """save_state after save_at steps of a user loop, the saved datasets as read back
    through read_state, a fresh solver's load_state + the remaining steps, and the first
    solver continued without interruption."""
    case = C.CASES[spec["base"]]
    n1, nt = spec["save_at"], case["Nt"]
    solver = make_solver(wakis, case, make_grid(wakis, case))
    beam = wakis.sources.Beam(**case["beam"])
    for n in range(n1):
        beam.update(solver, n * solver.dt)
        solver.one_step()
    solver.save_state("state.h5")
    st = solver.read_state("state.h5")
    keys = sorted(st.keys())
    saved = {k: np.array(st[k]) for k in keys}
    st.close()
    s2 = make_solver(wakis, case, make_grid(wakis, case))
    s2.load_state("state.h5")
    beam2 = wakis.sources.Beam(**case["beam"])
    for n in range(n1, nt):
        beam2.update(s2, n * s2.dt)
        s2.one_step()
    for n in range(n1, nt):
        beam.update(solver, n * solver.dt)
        solver.one_step()
    res = dict(keys=np.array(keys), dt=np.float64(solver.dt))
    for k, v in saved.items():
        res["saved_" + k] = v
    for k in ("E", "H", "J"):
        res["restart_" + k] = np.array(getattr(s2, k).toarray())  # copies: reset_fields zeroes in place
        res["cont_" + k] = np.array(getattr(solver, k).toarray())
    s2.reset_fields()
    res["reset_max"] = np.float64(max(np.abs(getattr(s2, k).toarray()).max() for k in ("E", "H", "J")))
    out[name] = res


def run_refine(wakis, out):
    """GridFIT3D.refine_axis of the reference on the seeded snap sets of REFINE_CASES, and
    the exception its 'subdivision' method raises."""
    g = wakis.GridFIT3D(0, 1, 0, 1, 0, 1, 2, 2, 2, verbose=0)
    res = {}
    for i, (seed, lo, hi, n, ns, method) in enumerate(C.REFINE_CASES):
        res[f"x{i}"] = g.refine_axis(lo, hi, n, C.refine_snaps(seed, lo, hi, ns), method=method)
    try:
        g.refine_axis(0.0, 1.0, 11, np.array([0.0, 0.37, 1.0]), method="subdivision")
        err = ("", "")
    except Exception as e:  # the reference's own failure is the fixture
        err = (type(e).__name__, str(e))
    res["subdivision_exc"] = np.array(err)
    out["refine_axis"] = res


def run_emsolve_save(wakis, out):
    """emsolve(save=True): the exception the reference raises and the files it leaves."""
    spec = C.EMSOLVE_SAVE_CASE
    g = spec["grid"]
    grid = wakis.GridFIT3D(g["xmin"], g["xmax"], g["ymin"], g["ymax"], g["zmin"], g["zmax"], g["Nx"], g["Ny"],
                           g["Nz"], verbose=0)
    solver = wakis.SolverFIT3D(grid, bc_low=["pec"] * 3, bc_high=["pec"] * 3, verbose=0)
    before = set(os.listdir("."))
    err = ("", "")
    try:
        solver.emsolve(spec["Nt"], save=True, fields=spec["fields"], components=spec["components"])
    except Exception as e:  # the reference's own failure is the fixture
        err = (type(e).__name__, str(e))
    files = sorted(set(os.listdir(".")) - before)
    out["emsolve_save"] = dict(exc_type=np.array(err[0]), exc_msg=np.array(err[1]), files=np.array(files),
                               nstep=np.int64(getattr(solver, "nstep", 0)))


def run_wakefile(wakis, name, case, out):
    """The reference's WakeSolver post-processing of a synthetic Ez file (written through
    the h5py stand-in), without a solver run."""
    import h5py  # the stand-in
    meta, slabs = C.synthetic_history(case["seed"], case["nz"], case["nt"], case["shape3"], case["t0"],
                                      case.get("side", 3))
    fname = os.path.join(os.getcwd(), name + "_Ez.h5")
    hf = h5py.File(fname, "w")
    for k, v in meta.items():
        hf[k] = v
    for n in range(len(slabs)):
        hf["#" + str(n).zfill(5)] = slabs[n]
    wake = wakis.WakeSolver(save=False, verbose=0, Ez_file=fname, **case["wake"])
    wake.n_transverse_cells = case.get("n_transverse_cells", 1)
    wake.solve(compute_plane=case["plane"])
    res = dict(s=wake.s, WP=wake.WP, f=wake.f, Z=wake.Z, lambdas=wake.lambdas,
               slab_sum=np.float64(np.sum(slabs)))
    if case["plane"] != "longitudinal":
        res.update(WP_3d=wake.WP_3d, WPx=wake.WPx, WPy=wake.WPy, Zx=wake.Zx, Zy=wake.Zy)
    out[name] = res


def test001_inputs(ref_root):
    """Golden vectors held by the reference's tests/test_001_pec_cubic_cavity.py, plus the
    STL bounds (the domain) parsed from tests/stl/001_cubic_cavity.stl."""
    sys.path.insert(0, os.path.join(ref_root, "tests"))
    import test_001_pec_cubic_cavity as t001
    cls = t001.TestPecCubicCavity
    src = open(os.path.join(ref_root, "tests", "test_001_pec_cubic_cavity.py")).read()
    wp_cs = float(re.search(r"np\.cumsum\(np\.abs\(wake\.WP\)\)\[-1\] == pytest\.approx\(\s*([0-9.eE+-]+)", src).group(1))
    z_cs = float(re.search(r"np\.cumsum\(np\.abs\(wake\.Z\)\)\[-1\] == pytest\.approx\(\s*([0-9.eE+-]+)", src).group(1))
    stl = open(os.path.join(ref_root, "tests", "stl", "001_cubic_cavity.stl")).read()
    v = np.array([[float(a) for a in ln.split()[1:4]] for ln in stl.splitlines() if ln.strip().startswith("vertex")])
    bounds = np.array([v[:, 0].min(), v[:, 0].max(), v[:, 1].min(), v[:, 1].max(), v[:, 2].min(), v[:, 2].max()])
    return dict(WP_samples=np.asarray(cls.WP, dtype=np.float64), Z_samples=np.asarray(cls.Z),
                WP_cumsum=wp_cs, Z_cumsum=z_cs, bounds=bounds)


def run_test001(wakis, inputs):
    """Reference FP32 run of the test_001 setup with the analytic corner-rule mask."""
    b = inputs["bounds"]
    Nx, Ny, Nz = 50, 50, 150
    grid = wakis.GridFIT3D(*b, Nx, Ny, Nz, verbose=0)
    tol = 1e-3 * min(np.min(grid.dx), np.min(grid.dy), np.min(grid.dz))
    m = C.test001_boxes_corner_rule(grid.x, grid.y, grid.z, tol)
    grid.stl_solids, grid.stl_materials, grid.stl_colors = {"cavity": "c"}, {"cavity": [1.0, 1.0]}, {"cavity": "b"}
    grid.grid["cavity"] = m.reshape(-1)
    wake = wakis.WakeSolver(wakelength=1.0, q=1e-9, sigmaz=18.5e-3, beta=1.0, xsource=0.0, ysource=0.0,
                            xtest=0.0, ytest=0.0, save=False, verbose=0,
                            Ez_file=os.path.join(os.getcwd(), "001_Ez.h5"), skip_cells=12)
    solver = wakis.SolverFIT3D(grid, wake, bc_low=["pec"] * 3, bc_high=["pec"] * 3, use_stl=True, bg="pec",
                               dtype=np.float32, verbose=0)
    solver.wakesolve(wakelength=1.0, save_J=False)
    return dict(Nt=solver.Nt, dt=np.float64(solver.dt), s=wake.s, WP=wake.WP, f=wake.f, Z=wake.Z,
                mask_count=int(m.sum()))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("reference")
    ap.add_argument("--test001", action="store_true")
    ap.add_argument("--only", default=None)
    a = ap.parse_args()
    ref_root = os.path.abspath(a.reference)
    wakis = load_reference(ref_root)
    out = {}
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as tmp:
        os.chdir(tmp)
        try:
            for name, case in C.CASES.items():
                if a.only and name != a.only:
                    continue
                print("case", name, flush=True)
                {"wake": run_wake, "emsolve": run_emsolve, "resonator": run_resonator,
                 "userloop": run_userloop}[case["kind"]](wakis, name, case, out)
            for name, case in C.WAKE_FILE_CASES.items():
                if a.only and name != a.only:
                    continue
                print("case", name, flush=True)
                run_wakefile(wakis, name, case, out)
            for name, spec in C.CHECKPOINT_CASES.items():
                if a.only and name != a.only:
                    continue
                print("case", name, flush=True)
                run_checkpoint(wakis, name, spec, out)
            if not a.only or a.only == "refine_axis":
                print("case refine_axis", flush=True)
                run_refine(wakis, out)
            if not a.only or a.only == "emsolve_save":
                print("case emsolve_save", flush=True)
                run_emsolve_save(wakis, out)
            if a.test001:
                inp = test001_inputs(ref_root)
                res = run_test001(wakis, inp)
                res.update(inp)
                out["test001"] = res
        finally:
            os.chdir(cwd)
    for name, res in out.items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **res)
        print("wrote", name, {k: np.shape(v) for k, v in res.items()})


if __name__ == "__main__":
    main()
