"""Runs the parity cases of tests/golden/cases.py through wakis_gb300 (the CUDA path),
returning dicts with the keys of the golden fixtures."""

import numpy as np
from scipy.constants import c as c_light

import cases as C


def make_grid(wg, case):
    x, y, z = C.axes(case)
    g = case["grid"]
    solids = C.solids_for(case)
    kw = {}
    if solids:
        kw = dict(stl_solids={n: m for n, m, _ in solids}, stl_materials={n: mat for n, _, mat in solids})
    if "x" in g:
        return wg.GridFIT3D(x=x, y=y, z=z, verbose=0, **kw)
    return wg.GridFIT3D(g["xmin"], g["xmax"], g["ymin"], g["ymax"], g["zmin"], g["zmax"], g["Nx"], g["Ny"], g["Nz"],
                        verbose=0, **kw)


def make_solver(wg, case, grid, wake=None, dtype=None, dt=None):
    dty = dtype or (np.float32 if case["dtype"] == "float32" else np.float64)
    return wg.SolverFIT3D(grid, wake, cfln=case.get("cfln", 0.5), dt=dt, bc_low=list(case["bc_low"]),
                          bc_high=list(case["bc_high"]), use_stl=bool(case.get("solids")), bg=case["bg"], dtype=dty,
                          n_pml=case.get("n_pml", 10), verbose=0)


def run_case(name, case=None, tmpdir=".", userloop_wake=False, dtype=None, dt=None):
    import wakis_gb300 as wg
    case = case or C.CASES[name]
    kind = case["kind"]
    if kind == "resonator":
        N = case["N"]
        d = 1.0 / N
        grid = wg.GridFIT3D(-0.5 + d / 2, 0.5 + d / 2, -0.5 + d / 2, 0.5 + d / 2, -0.5 + d / 2, 0.5 + d / 2, N, N, N,
                            verbose=0)
        s = wg.SolverFIT3D(grid, bc_low=["pec"] * 3, bc_high=["pec"] * 3, verbose=0, dtype=dtype or np.float64)
        Hx, Hy, Hz, _ = C.resonator_H(N, s.dt)
        s.H[:, :, :, "x"] = Hx
        s.H[:, :, :, "y"] = Hy
        s.H[:, :, :, "z"] = Hz
        ey = []
        for _ in range(case["Nt"]):
            ey.append(s.E[N // 2, N // 2, N // 2, "y"])
            s.one_step()
        return dict(dt=np.float64(s.dt), Ey=np.array(ey), E=s.E.numpy(), H=s.H.numpy())
    grid = make_grid(wg, case)
    if kind == "wake":
        wake = wg.WakeSolver(wakelength=case["wakelength"], save=False, verbose=0, results_folder=str(tmpdir),
                             **case["wake"])
        s = make_solver(wg, case, grid, wake, dtype, dt)
        s.logger.wakeSolver["results_folder"] = str(tmpdir)
        mon = wg.FieldMonitor(case["monitor"]) if "monitor" in case else None
        cb = (lambda sv, t: None) if userloop_wake else None
        s.wakesolve(wakelength=case["wakelength"], compute_plane=case["compute_plane"], callback=cb,
                    use_field_monitor=mon is not None, field_monitor=mon)
        res = dict(Nt=s.Nt, dt=np.float64(s.dt), s=wake.s, WP=wake.WP, f=wake.f, Z=wake.Z, lambdas=wake.lambdas,
                   E=s.E.numpy(), H=s.H.numpy(), J=s.J.numpy())
        if mon is not None:
            res.update({k + "_acc": v.cpu().numpy() for k, v in mon.get_components().items()})
        if case["compute_plane"] != "longitudinal":
            res.update(WP_3d=wake.WP_3d, WPx=wake.WPx, WPy=wake.WPy, Zx=wake.Zx, Zy=wake.Zy)
        return res
    s = make_solver(wg, case, grid, dtype=dtype, dt=dt)
    if kind == "userloop":
        beam = wg.sources.Beam(**case["beam"])
        for n in range(case["Nt"]):
            beam.update(s, n * s.dt)
            s.one_step()
        return dict(dt=np.float64(s.dt), E=s.E.numpy(), H=s.H.numpy(), J=s.J.numpy())
    src = None
    sc = case.get("source")
    if sc is not None and sc["type"] == "PlaneWave":
        f = sc["f_nodes"] / ((s.z.max() - s.z.min()) / c_light)
        src = wg.sources.PlaneWave(xs=slice(*sc["xs"]), ys=slice(*sc["ys"]), zs=sc["zs"], beta=sc["beta"],
                                   amplitude=sc["amplitude"], f=f, nodes=sc["nodes"], phase=sc["phase"])
        if case.get("dt_override") == "1/f/200":
            s.dt = 1 / f / 200
    elif sc is not None and sc["type"] == "WavePacket":
        src = wg.sources.WavePacket(zs=sc["zs"], sigmaz=sc["sigmaz"], sigmaxy=sc["sigmaxy"],
                                    wavelength=sc["wavelength"], amplitude=sc["amplitude"])
    elif sc is not None:
        src = C.point_source(wg, sc)
    if "random_init" in case:
        E0, H0 = C.random_fields(s.N, case["random_init"], np.dtype(s.dtype))
        s.E.fromarray(E0)
        s.H.fromarray(H0)
    probes = []
    cb = None
    if "probes" in case:
        P = C.probe_points(case)

        def cb(sv, t):
            probes.append([sv.E[int(i), int(j), int(k), "z"] for i, j, k in P])
    s.emsolve(case["Nt"], source=src, callback=cb)
    res = dict(dt=np.float64(s.dt), E=s.E.numpy(), H=s.H.numpy(), J=s.J.numpy())
    if probes:
        res["probes"] = np.array(probes, dtype=np.float64)
    return res


def run_wake_partial(case, nsteps, tmpdir=".", dtype=None, dt=None):
    """The first ``nsteps`` steps of a wake run through the CUDA path: the tap table of
    the full run is installed and the device loop is stopped after nsteps steps, so the
    device accumulators hold the partial line sums (taps with time index < nsteps).
    Returns s, dt, Nt (of the full run), WP_3d (9, len(s)), E and H."""
    import wakis_gb300 as wg
    grid = make_grid(wg, case)
    wake = wg.WakeSolver(wakelength=case["wakelength"], save=False, verbose=0, results_folder=str(tmpdir),
                         **case["wake"])
    s = make_solver(wg, case, grid, wake, dtype, dt)
    beam, Nt = s._wake_prepare(wake, case["wakelength"], "both")
    vt = s._wake_device_setup(beam, Nt)
    first = s._wake_first_step(beam)
    s._device_steps(first, nsteps - first)
    s._wake_device_done(vt[:nsteps], nsteps)
    sv, wp3d, _, _ = wake._finalize_device()
    return dict(s=sv, dt=np.float64(s.dt), Nt=Nt, WP_3d=wp3d, E=s.E.numpy(), H=s.H.numpy())
