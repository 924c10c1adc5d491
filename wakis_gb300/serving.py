"""Served wake solves: continuous batching of cavity wakefield requests on one GPU.

There is no counterpart in the reference: Wakis runs one ``SolverFIT3D.wakesolve``
(wakis/routines.py:231-485) per process.  This module keeps that call's inputs and
outputs per request -- a ``GridFIT3D`` + ``WakeSolver`` + ``SolverFIT3D`` and the
resulting ``WakeSolver.WP / WPx / WPy / Z / Zx / Zy`` -- and runs many requests through
one ``libwakis_fit`` pool (``FitPool``), which steps all admitted grids together.

Flow of a request:

1. it arrives and waits in a queue;
2. it is admitted when its device footprint (``footprint_bytes``) fits in the pool's
   memory budget, and its solver is built: host setup, then the coefficient build and
   the first step on the GPU;
3. the pool takes its remaining steps in batched chunks, next to every other admitted
   request; requests join and leave between chunks;
4. when the pool reports it done, the wake potential is combined and the impedance is
   taken (FP64, on the device); its memory is freed and released from the budget.

Time-to-impedance is measured from arrival to the impedance on the host.
"""

import collections
import dataclasses
import math
import tempfile
import time

import numpy as np

from . import _native as nat

MM = 1e-3


@dataclasses.dataclass
class CavityRequest:
    """One wakefield solve of a cube cavity with a beam pipe (the geometry of the 60x60x120
    cavity wake run, scaled): vacuum = {|x|,|y|,|z| <= side/2} U {x^2 + y^2 <= rp^2}, domain
    x, y in [-0.6 side, 0.6 side], z in [-1.2 side, 1.2 side], n x n x 2n cells.
    sigma == 0: PEC walls (background PEC, ABC at the z ends, CFL 1.0).  sigma > 0: lossy
    walls [1, 1, sigma] (relaxation form), 10-cell PML at the z ends, CFL 0.5 (the
    explicit loss term is unstable at CFL 1.0)."""
    tag: int
    side: float
    rp: float
    n: int
    sigmaz: float
    sigma: float
    arrival: float = 0.0
    wakelength: float = 1.0
    q: float = 1e-9
    fmax: float = 5e9

    @property
    def cells(self):
        return self.n * self.n * 2 * self.n

    @property
    def lossy(self):
        return self.sigma > 0


def cavity_sweep_requests(count=64, seed=3, rate_hz=None, wakelength=1.0):
    """The serving sweep's instances, drawn from numpy.random.default_rng(seed): cube side
    U(20, 60) mm, pipe radius U(3, 8) mm, cells per transverse dimension uniform in
    48..160 (z twice that), sigma_z U(5, 15) mm, walls PEC or lossy with sigma U(1e3, 1e6)
    S/m (equal odds).  Arrivals form a Poisson stream of rate rate_hz (all at t = 0 when
    rate_hz is None)."""
    rng = np.random.default_rng(seed)
    out = []
    t = 0.0
    for i in range(count):
        side = rng.uniform(20, 60) * MM
        rp = rng.uniform(3, 8) * MM
        n = int(rng.integers(48, 161))
        sigmaz = rng.uniform(5, 15) * MM
        lossy = bool(rng.integers(0, 2))
        sigma = float(rng.uniform(1e3, 1e6)) if lossy else 0.0
        if rate_hz:
            t += float(rng.exponential(1.0 / rate_hz))
        out.append(CavityRequest(tag=i, side=side, rp=rp, n=n, sigmaz=sigmaz, sigma=sigma, arrival=t,
                                 wakelength=wakelength))
    return out


def footprint_bytes(req, dtype=np.float32, kernels="direct"):
    """Device bytes a request holds while it is served: E, H, J (3 x 3N field words), the
    FP64 material tensors ieps, imu, sigma (3 x 3N x 8), the library's coefficient arrays
    (ch, ce and, with losses, cl: 3N field words each) and their 2-byte codes, with the
    fused step the second E and H buffers (6N field words), the cell mask and a fixed
    allowance for the 1-D metrics, tap tables, the code table and allocator rounding."""
    N = req.cells
    w = np.dtype(dtype).itemsize
    ncoef = 3 if req.lossy else 2
    fused = kernels == "fused" or (kernels == "auto" and req.n % 2 == 0)
    return int(N * (9 * w + 72 + 3 * w * ncoef + 1 + 2 + (6 * w if fused else 0)) + 8 * 2 ** 20)


def _axes(req):
    h, hz = 0.6 * req.side, 1.2 * req.side
    return (np.linspace(-h, h, req.n + 1), np.linspace(-h, h, req.n + 1), np.linspace(-hz, hz, 2 * req.n + 1))


def _vacuum_mask(req, device):
    import torch
    x, y, z = _axes(req)
    xc, yc, zc = (torch.as_tensor(a[:-1] + np.diff(a) / 2, device=device) for a in (x, y, z))
    X, Y, Z = xc[:, None, None], yc[None, :, None], zc[None, None, :]
    half = req.side / 2
    cube = (X.abs() <= half) & (Y.abs() <= half) & (Z.abs() <= half)
    return cube | (X ** 2 + Y ** 2 <= req.rp ** 2)


def cfl_dt(req, dtype=np.float32):
    """The time step SolverFIT3D takes for the request, rounded to dtype (the solver's own
    formula, wakis/solverFIT3D.py:294-307).  An FP64 solve given the FP32 step is the
    FP64 reference of an FP32 solve: both then sample the wake at the same times."""
    from scipy.constants import c as c_light
    x, y, z = _axes(req)
    cfln = 0.5 if req.lossy else 1.0
    dt = cfln / (c_light * np.sqrt(1 / np.min(np.diff(x)) ** 2 + 1 / np.min(np.diff(y)) ** 2
                                   + 1 / np.min(np.diff(z)) ** 2))
    return float(np.dtype(dtype).type(dt))


def build(req, dtype=np.float32, device=0, results_folder=None, dt=None):
    """GridFIT3D, WakeSolver and SolverFIT3D of a request (cell-centre masks)."""
    import torch
    from .gridFIT3D import GridFIT3D
    from .solverFIT3D import SolverFIT3D
    from .wakeSolver import WakeSolver
    dev = torch.device("cuda", device)
    x, y, z = _axes(req)
    vac = _vacuum_mask(req, dev)
    if req.lossy:
        grid = GridFIT3D(x=x, y=y, z=z, stl_solids={"walls": ~vac}, stl_materials={"walls": [1.0, 1.0, req.sigma]},
                         verbose=0)
        bc, bg, cfln = ["pec", "pec", "pml"], [1.0, 1.0], 0.5
    else:
        grid = GridFIT3D(x=x, y=y, z=z, stl_solids={"cavity": vac}, stl_materials={"cavity": "vacuum"}, verbose=0)
        bc, bg, cfln = ["pec", "pec", "abc"], "pec", 1.0
    del vac
    wake = WakeSolver(wakelength=req.wakelength, q=req.q, sigmaz=req.sigmaz, beta=1.0, xsource=0.0, ysource=0.0,
                      xtest=0.0, ytest=0.0, fmax=req.fmax, save=False, verbose=0,
                      results_folder=results_folder or tempfile.gettempdir())
    solver = SolverFIT3D(grid, wake, cfln=cfln, dt=dt, bc_low=bc, bc_high=bc, use_stl=True, bg=bg, dtype=dtype,
                         n_pml=10, verbose=0)
    return grid, wake, solver


class ServedSolve:
    """A request's solver between admission and its impedance."""

    def __init__(self, req, dtype=np.float32, device=0, results_folder=None, kernels="direct"):
        self.req = req
        self.grid, self.wake, self.solver = build(req, dtype, device, results_folder)
        s = self.solver
        # 'direct': the pool's two-pass kernels; 'fused' (or 'auto' with Nx even): the
        # pool's fused step on plane segments (coded coefficients, Nx <= 256; any other
        # grid takes the two-pass kernels), which also holds the second E, H buffers
        s.kernels = kernels
        self.beam, self.Nt = s._wake_prepare(self.wake, req.wakelength, "both")
        self.vt = s._wake_device_setup(self.beam, self.Nt)
        self.first = s._wake_first_step(self.beam)
        if s.step_0:
            s._set_ghosts_to_0()
            s.step_0 = False
        s._sync_coeffs()
        s._ensure_codes()  # the pool's two-pass classes read the coefficient codes

    def submit(self, pool):
        pool.submit(self.solver._ctx, self.first, self.Nt - self.first, self.req.tag)

    def finish(self):
        s = self.solver
        s._run_steps += self.Nt - self.first
        s._wake_device_done(self.vt, self.Nt)
        self.wake.solve(compute_plane="both")
        w = self.wake
        return dict(s=w.s, WP=w.WP, WPx=w.WPx, WPy=w.WPy, f=w.f, Z=w.Z, Zx=w.Zx, Zy=w.Zy)

    def close(self):
        self.solver._ctx.close()
        self.solver = self.wake = self.grid = self.beam = None


def solve_alone(req, dtype=np.float32, device=0, dt=None, kernels="auto"):
    """The request through the plain public API (SolverFIT3D.wakesolve), one at a time.
    kernels='direct' runs the two-pass kernels, whose per-cell code the pool shares (the
    pooled result then equals this one bit for bit)."""
    grid, wake, solver = build(req, dtype, device, dt=dt)
    solver.kernels = kernels
    solver.wakesolve(wakelength=req.wakelength, compute_plane="both")
    out = dict(s=wake.s, WP=wake.WP, WPx=wake.WPx, WPy=wake.WPy, f=wake.f, Z=wake.Z, Zx=wake.Zx, Zy=wake.Zy,
               Nt=solver.Nt, cells=req.cells)
    solver._ctx.close()
    return out


POOL_VARIANTS = {4: (2, 3), 2: (3, 4), 1: (3, 4)}
POOL_FUSED_VARIANTS = {4: (2, 3), 2: (3, 4), 1: (3, 4)}  # the pooled fused kernel's compiled budgets


def run_resident(pool, reqs, kernels="direct"):
    """Builds every request, submits them together and waits: returns (cell-updates,
    seconds of pool time with chunks in flight, jobs)."""
    jobs = [ServedSolve(r, kernels=kernels) for r in reqs]
    busy0 = pool.stats()["busy_ms"]
    for j in jobs:
        j.submit(pool)
    done = []
    while len(done) < len(jobs):
        done += pool.poll(wait_ms=50)
    if any(d["status"] != 0 for d in done):
        raise nat.FitError(min(d["status"] for d in done), "pooled calibration solve failed")
    busy = (pool.stats()["busy_ms"] - busy0) / 1e3
    return sum(j.req.cells * (j.Nt - j.first) for j in jobs), busy, jobs


def calibration_requests(seed=11, per_class=4, wakelength=0.1):
    """Grids of the serving sweep's distribution (cavity_sweep_requests' ranges) with Nx forced
    into each vector-width class: per class, per_class requests, half of them lossy."""
    rng = np.random.default_rng(seed)
    out = {}
    tag = 10000
    for vec in (4, 2, 1):
        reqs = []
        for i in range(per_class):
            n = int(rng.integers(48, 157))
            n = n - n % 4 + {4: 0, 2: 2, 1: 1}[vec]
            reqs.append(CavityRequest(tag=tag, side=rng.uniform(20, 60) * MM, rp=rng.uniform(3, 8) * MM, n=n,
                                      sigmaz=rng.uniform(5, 15) * MM, sigma=(float(rng.uniform(1e3, 1e6)) if i % 2
                                                                               else 0.0), wakelength=wakelength))
            tag += 1
        out[vec] = reqs
    return out


def autotune(pool, calib=None, repeats=1, kernels="direct"):
    """Per vector-width class, times every compiled variant of the pool's kernels on
    calibration grids (all resident at once, pool time only) and keeps the fastest:
    the two-pass kernels with kernels='direct', the fused step with kernels='fused'.
    Returns {vec: {"choice": ctas_per_sm, "rates": {variant: cell-updates/s}}}."""
    import torch
    calib = calib or calibration_requests()
    fused = kernels == "fused"
    select = pool.tune_fused if fused else pool.tune
    out = {}
    for vec, reqs in calib.items():
        rates = {}
        for minb in (POOL_FUSED_VARIANTS if fused else POOL_VARIANTS)[vec]:
            select(vec, minb)
            best = 0.0
            for _ in range(repeats):
                cu, busy, jobs = run_resident(pool, reqs, kernels=kernels)
                for j in jobs:
                    j.close()
                del jobs
                torch.cuda.empty_cache()
                best = max(best, cu / busy if busy > 0 else 0.0)
            rates[minb] = best
        choice = max(rates, key=rates.get)
        select(vec, choice)
        out[vec] = {"choice": choice, "rates": rates}
    return out


def _percentile(v, p):
    return float(np.percentile(np.asarray(v, dtype=np.float64), p)) if len(v) else None


def summarize(records, makespan_s):
    tti = [r["tti_s"] for r in records]
    cells = sum(r["cells"] * r["steps"] for r in records)
    return {"solves": len(records), "makespan_s": makespan_s,
            "solves_per_hour": len(records) / makespan_s * 3600 if makespan_s > 0 else None,
            "tti_p50_s": _percentile(tti, 50), "tti_p99_s": _percentile(tti, 99), "tti_max_s": max(tti) if tti else None,
            "mcell_updates_per_s": cells / makespan_s / 1e6 if makespan_s > 0 else None}


class Admission:
    """First-fit admission in arrival order with bounded bypass.

    ``admit(queue, size, reserve)`` walks the waiting requests oldest first and admits
    (removes from ``queue`` and yields with its size) every request for which
    ``reserve(size(req))`` succeeds.  A request admitted while an older one keeps waiting
    counts as a bypass of the oldest; after ``max_bypass`` of them only the oldest may be
    admitted, so a large request waits for at most that many smaller ones."""

    def __init__(self, max_bypass=8):
        self.max_bypass = max_bypass
        self.bypass = 0
        self._head = None

    def admit(self, queue, size, reserve):
        i = 0
        while i < len(queue):
            if queue[0] is not self._head:
                self._head = queue[0]
                self.bypass = 0
            if i > 0 and self.bypass >= self.max_bypass:
                return
            req = queue[i]
            nbytes = size(req)
            if not reserve(nbytes):
                i += 1
                continue
            queue.pop(i)
            if i > 0:
                self.bypass += 1
            yield req, nbytes


class ServingLoop:
    """Continuous batching of requests through one FitPool.

    Admission is first-fit in arrival order: a request that fits the free budget is
    admitted even when an earlier one does not, unless the oldest waiting request has
    already been passed over ``max_bypass`` times, after which admission is strict FIFO
    until it gets in (bounded waiting for large requests).

    A failure ends one request, never the loop: a request whose footprint exceeds the
    whole budget is rejected on arrival, one whose solver cannot be built (out of memory,
    a library error) fails at admission, one cancelled while queued or running
    (``cancel``) is handed back by the pool, and one whose wake potential or impedance is
    not finite when read back fails at completion.  Each ends as a record with a status
    ('done', 'rejected', 'failed', 'cancelled') and a reason; the others run on.  With
    ``trace_path`` every record is also appended to that file as one JSON line."""

    def __init__(self, budget_bytes, chunk_steps=64, ctas_per_sm=0, device=0, dtype=np.float32, max_bypass=8,
                 keep_results=True, variants=None, kernels="direct", trace_path=None, fused_variants=None):
        self.budget = int(budget_bytes)
        self.pool = nat.Pool(budget_bytes, chunk_steps=chunk_steps, ctas_per_sm=ctas_per_sm, device=device)
        for vec, minb in (variants or {}).items():
            self.pool.tune(vec, minb)
        for vec, minb in (fused_variants or {}).items():
            self.pool.tune_fused(vec, minb)
        self.device = device
        self.dtype = dtype
        self.kernels = kernels
        self.admission = Admission(max_bypass)
        self.keep_results = keep_results
        self.results = {}
        self.trace_path = trace_path
        self._cancel = set()

    def close(self):
        self.pool.close()

    def cancel(self, tag):
        """Cancels a request: before admission it is dropped from the queue, while it runs
        the pool stops stepping it.  Takes effect in the loop's next iteration."""
        self._cancel.add(tag)

    def _trace(self, rec):
        if self.trace_path:
            import json
            with open(self.trace_path, "a") as fh:
                fh.write(json.dumps(rec) + "\n")

    def run(self, requests, time_scale=1.0, on_tick=None, readback_hook=None):
        """Serves the requests (arrival times in seconds, scaled by time_scale) and returns
        per-request records and a summary of the completed ones.  on_tick(loop, now_s, running_tags)
        runs once per loop iteration (a caller can cancel from it); readback_hook(tag,
        result) may inspect or alter a finished request's host-side results before the
        finiteness check."""
        tmp = tempfile.mkdtemp()
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        queue = []
        running = {}
        records = []
        t0 = time.perf_counter()
        size = lambda r: footprint_bytes(r, self.dtype, self.kernels)

        def record(req, status, reason="", **kw):
            rec = dict(tag=req.tag, status=status, reason=reason, cells=req.cells, lossy=req.lossy,
                       arrival_s=req.arrival * time_scale, end_s=time.perf_counter() - t0)
            rec.update(kw)
            records.append(rec)
            self._trace(rec)

        while pending or queue or running:
            now = time.perf_counter() - t0
            while pending and pending[0].arrival * time_scale <= now:
                req = pending.popleft()
                if size(req) > self.budget:
                    record(req, "rejected", "footprint above the pool budget", footprint=size(req))
                else:
                    queue.append(req)
            if on_tick is not None:
                on_tick(self, now, sorted(running))
            for req in [r for r in queue if r.tag in self._cancel]:
                queue.remove(req)
                self._cancel.discard(req.tag)
                record(req, "cancelled", "cancelled before admission")
            for tag in [t for t in running if t in self._cancel]:
                self._cancel.discard(tag)
                try:
                    self.pool.cancel(tag)
                except nat.FitError:  # it finished in the meantime; poll reports it
                    pass
            admitted = False
            for req, nbytes in self.admission.admit(queue, size, self.pool.reserve):
                t_adm = time.perf_counter() - t0
                try:
                    job = ServedSolve(req, self.dtype, self.device, tmp, self.kernels)
                    job.submit(self.pool)
                except (nat.FitError, RuntimeError) as e:  # a library error or torch's out-of-memory
                    self.pool.release(nbytes)
                    record(req, "failed", f"setup: {e}", admitted_s=t_adm, footprint=nbytes)
                    continue
                running[req.tag] = (job, nbytes, t_adm, time.perf_counter() - t0)
                admitted = True
            if running:
                if queue and not admitted:
                    wait = 50
                elif pending:
                    wait = max(0, min(50, int((pending[0].arrival * time_scale - (time.perf_counter() - t0)) * 1e3)))
                else:
                    wait = 50
                for d in self.pool.poll(wait_ms=wait):
                    job, nbytes, t_adm, t_sub = running.pop(d["tag"])
                    req = job.req
                    times = dict(admitted_s=t_adm, submitted_s=t_sub, pool_submit_ms=d["t_submit_ms"],
                                 pool_start_ms=d["t_start_ms"], pool_done_ms=d["t_done_ms"], footprint=nbytes)
                    if d["status"] == nat.FIT_ERR_CANCELLED:
                        record(req, "cancelled", "cancelled while running", **times)
                    elif d["status"] != 0:
                        record(req, "failed", f"pool status {d['status']}", **times)
                    else:
                        res = job.finish()
                        if readback_hook is not None:
                            readback_hook(req.tag, res)
                        bad = [k for k in ("WP", "WPx", "WPy", "Z", "Zx", "Zy")
                               if not np.all(np.isfinite(np.asarray(res[k])))]
                        t_done = time.perf_counter() - t0
                        if bad:
                            record(req, "failed", "non-finite " + ", ".join(bad), steps=job.Nt, **times)
                        else:
                            record(req, "done", steps=job.Nt, done_s=t_done, tti_s=t_done - req.arrival * time_scale,
                                   pool_ms=d["t_done_ms"] - d["t_submit_ms"], **times)
                            if self.keep_results:
                                self.results[req.tag] = res
                    job.close()
                    del job
                    self.pool.release(nbytes)
            elif pending and not queue:
                time.sleep(max(0.0, pending[0].arrival * time_scale - (time.perf_counter() - t0)))
        makespan = time.perf_counter() - t0
        out = summarize([r for r in records if r["status"] == "done"], makespan)
        out["failed"] = {st: sum(r["status"] == st for r in records) for st in ("rejected", "failed", "cancelled")}
        out["pool"] = self.pool.stats()
        return records, out


def serve_one_at_a_time(requests, dtype=np.float64, device=0, time_scale=1.0, dt_of=None, keep=None):
    """Baseline: the same requests through SolverFIT3D.wakesolve one at a time (a single
    server queue in arrival order), for time-to-impedance and solves/hour.  dt_of(req)
    gives each solve's time step (None: the solver's own); keep, a dict, receives each
    request's results by tag."""
    import torch
    reqs = sorted(requests, key=lambda r: r.arrival)
    records = []
    t0 = time.perf_counter()
    for req in reqs:
        now = time.perf_counter() - t0
        if req.arrival * time_scale > now:
            time.sleep(req.arrival * time_scale - now)
        t_start = time.perf_counter() - t0
        out = solve_alone(req, dtype, device, dt=dt_of(req) if dt_of else None)
        torch.cuda.synchronize(device)
        if keep is not None:
            keep[req.tag] = out
        t_done = time.perf_counter() - t0
        records.append(dict(tag=req.tag, cells=req.cells, steps=out["Nt"], lossy=req.lossy,
                            arrival_s=req.arrival * time_scale, admitted_s=t_start, done_s=t_done,
                            tti_s=t_done - req.arrival * time_scale))
        del out
        torch.cuda.empty_cache()
    return records, summarize(records, time.perf_counter() - t0)


def poisson_rate_for(requests, budget_bytes, service_rate_cells_per_s, dtype=np.float32, load=1.5):
    """An arrival rate at which admission by memory binds: requests arrive `load` times
    faster than the GPU clears them, so the queue grows and the budget decides how many
    run at once."""
    work = np.mean([r.cells * _steps_estimate(r) for r in requests])
    return load * service_rate_cells_per_s / work


def _steps_estimate(req):
    from scipy.constants import c as c_light
    d = 1.2 * req.side / req.n
    cfl = 0.5 if req.lossy else 1.0
    dt = cfl / (c_light * math.sqrt(3.0 / d ** 2))
    ti = 8.548921333333334 * req.sigmaz / c_light
    return (req.wakelength + ti * c_light + 2.4 * req.side) / c_light / dt
