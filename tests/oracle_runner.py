"""Runs the parity cases of tests/golden/cases.py through the CPU oracle.

Test infrastructure: the result dicts have the same keys as the golden fixtures that
make_golden.py writes from the reference, so a test can pin the oracle against the
reference and then compare the CUDA path with the oracle.
"""

import os
import sys

import numpy as np
from scipy.constants import c as c_light

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
if GOLDEN not in sys.path:
    sys.path.insert(0, GOLDEN)

import cases as C  # noqa: E402
from oracle import fit_oracle as O  # noqa: E402


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def oracle_solver(case):
    x, y, z = C.axes(case)
    g = O.OracleGrid(x, y, z)
    dtype = np.float32 if case["dtype"] == "float32" else np.float64
    solids = [(m, mat) for _, m, mat in C.solids_for(case)]
    return O.OracleSolver(g, case["bc_low"], case["bc_high"], solids=solids, bg=case["bg"],
                          cfln=case.get("cfln", 0.5), dtype=dtype, n_pml=case.get("n_pml", 10))


class _ORACLE_SOURCES:
    """The oracle's point sources under the names the case descriptions use."""
    class sources:
        Dipole = O.OracleDipole
        Pulse = O.OraclePulse


def run_oracle_case(name, case=None):
    case = case or C.CASES[name]
    kind = case["kind"]
    if kind == "resonator":
        N = case["N"]
        d = 1.0 / N
        ax = np.linspace(-0.5 + d / 2, 0.5 + d / 2, N + 1)
        s = O.OracleSolver(O.OracleGrid(ax, ax, ax), ["pec"] * 3, ["pec"] * 3)
        Hx, Hy, Hz, _ = C.resonator_H(N, s.dt)
        for di, h in enumerate((Hx, Hy, Hz)):
            s.comp(s.H, di)[...] = h
        ey = []
        for _ in range(case["Nt"]):
            ey.append(s.comp(s.E, 1)[N // 2, N // 2, N // 2])
            s.one_step()
        return dict(dt=np.float64(s.dt), Ey=np.array(ey), E=s.E.copy(), H=s.H.copy())
    s = oracle_solver(case)
    if kind == "wake":
        wake = O.OracleWake(wakelength=case["wakelength"], **case["wake"])
        mon = O.OracleFieldMonitor(case["monitor"]) if "monitor" in case else None
        O.wakesolve(s, wake, case["wakelength"], case["compute_plane"], field_monitor=mon)
        res = dict(Nt=s.Nt, dt=np.float64(s.dt), s=wake.s, WP=wake.WP, f=wake.f, Z=wake.Z,
                   lambdas=wake.lambdas, E=s.E.copy(), H=s.H.copy(), J=s.J.copy())
        if mon is not None:
            res.update(Ex_acc=mon.Ex_acc, Ey_acc=mon.Ey_acc, Ez_acc=mon.Ez_acc)
        if case["compute_plane"] != "longitudinal":
            res.update(WP_3d=wake.WP_3d, WPx=wake.WPx, WPy=wake.WPy, Zx=wake.Zx, Zy=wake.Zy)
        return res
    if kind == "userloop":
        beam = O.OracleBeam(**case["beam"])
        for n in range(case["Nt"]):
            beam.update(s, n * s.dt)
            s.one_step()
        return dict(dt=np.float64(s.dt), E=s.E.copy(), H=s.H.copy(), J=s.J.copy())
    # emsolve
    src = None
    sc = case.get("source")
    if sc is not None and sc["type"] == "PlaneWave":
        f = sc["f_nodes"] / ((s.z.max() - s.z.min()) / c_light)
        src = O.OraclePlaneWave(xs=slice(*sc["xs"]), ys=slice(*sc["ys"]), zs=sc["zs"], beta=sc["beta"],
                                amplitude=sc["amplitude"], f=f, nodes=sc["nodes"], phase=sc["phase"])
        if case.get("dt_override") == "1/f/200":
            s.dt = 1 / f / 200
    elif sc is not None and sc["type"] == "WavePacket":
        src = O.OracleWavePacket(zs=sc["zs"], sigmaz=sc["sigmaz"], sigmaxy=sc["sigmaxy"],
                                 wavelength=sc["wavelength"], amplitude=sc["amplitude"])
    elif sc is not None:
        src = C.point_source(_ORACLE_SOURCES, sc)
    if "random_init" in case:
        E0, H0 = C.random_fields(s.N, case["random_init"], s.E.dtype)
        s.E[:] = E0
        s.H[:] = H0
    probes = []
    cb = None
    if "probes" in case:
        P = C.probe_points(case)

        def cb(sv, t):
            probes.append([sv.comp(sv.E, 2)[i, j, k] for i, j, k in P])
    O.emsolve(s, case["Nt"], source=src, callback=cb)
    res = dict(dt=np.float64(s.dt), E=s.E.copy(), H=s.H.copy(), J=s.J.copy())
    if probes:
        res["probes"] = np.array(probes, dtype=np.float64)
    return res


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.linalg.norm(b.ravel())
    num = np.linalg.norm((a - b).ravel())
    return num / den if den > 0 else num


def run_oracle_wake_partial(case, nsteps):
    """The first ``nsteps`` steps of a wake run through the oracle: the fields after them
    and the partial wake integral, i.e. the line sums over the taps whose time index is
    below nsteps (the tap table of the full run), combined across the 3x3 lines with the
    reference's non-reset accumulator.  Returns s, dt, Nt (of the full run), WP_3d
    (9, len(s)), E and H."""
    s = oracle_solver(case)
    wake = O.OracleWake(wakelength=case["wakelength"], **case["wake"])
    ixt = np.abs(s.x - wake.xtest).argmin()
    iyt = np.abs(s.y - wake.ytest).argmin()
    xx, yy = slice(ixt - 1, ixt + 2), slice(iyt - 1, iyt + 2)
    z = s.z
    tmax = (wake.wakelength + wake.ti * wake.v + (z.max() - z.min())) / wake.v
    Nt = int(tmax / s.dt)
    beam = O.OracleBeam(q=wake.q, sigmaz=wake.sigmaz, beta=wake.beta, xsource=wake.xsource, ysource=wake.ysource)
    ez = s.comp(s.E, 2)
    slabs = []
    for n in range(nsteps):
        beam.update(s, n * s.dt)
        slabs.append(np.array(ez[xx, yy, :], dtype=np.float64))
        s.one_step()
    slabs = np.array(slabs)
    wake.t = np.arange(0, Nt * s.dt, s.dt)
    wake.zf = z.copy()
    wake.dz = s.dz
    sv, it, valid, zz, nt = O.wp_index_table(wake, Nt)
    fed = valid & (it < nsteps)
    dzz = np.asarray(wake.dz, dtype=np.float64)
    kk = np.broadcast_to(np.arange(it.shape[1]), it.shape)
    wp = np.zeros_like(sv)
    wp3d = np.zeros((9, len(sv)))
    for li, (i, j) in enumerate((i, j) for i in range(-1, 2) for j in range(-1, 2)):
        ezt = slabs[:, 1 + i, 1 + j, zz].T  # (nz, nsteps)
        terms = np.where(fed, ezt[kk, np.where(fed, it, 0)] * dzz[kk], 0.0)
        wp = O._seq_rows(terms, start=wp) / (wake.q * 1e12)
        wp3d[li] = wp
    return dict(s=sv, dt=np.float64(s.dt), Nt=Nt, WP_3d=wp3d, E=s.E.copy(), H=s.H.copy())


def run_oracle_probes(case, nsteps):
    """emsolve of an emsolve case for ``nsteps`` steps through the oracle with E_z recorded
    at the case's probe points after every step; returns dt, probes (nsteps, P), E, H."""
    return run_oracle_case(None, case=dict(case, Nt=nsteps))
