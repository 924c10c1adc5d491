"""Benchmark of the FIT leapfrog hot path on GB300.

Workload (default): the large single-domain roofline run -- lossy pillbox cavity
(radius 50 mm, length 100 mm, wall sigma = 5.8e7 S/m in the relaxation form) with a
10 mm beam pipe to z = +-200 mm on a 512 x 512 x 1024 grid (268 M cells), FP32 fields,
16-cell PML at both z ends, Gaussian beam beta = 1, sigma_z = 5 mm, 3x3 wake taps active.

A "step" is one leapfrog step of the whole grid (prologue with the wake taps, then the
fused step -- or the H and E passes -- with the beam current), replayed from CUDA graphs
with the step number on the device: the loop wakesolve runs.  Inputs are far larger
than L2 (14 GB per step with coded coefficients, 22 GB dense), so no L2 flush is needed
between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  value = Mcell-updates/s (cells x steps / device time) with the
fields resident in HBM; e2e = the same metric for a complete wakesolve through the
public API (host geometry in, wake potential and impedance out, every host<->device
copy inside the timed region); roofline = the dominant kernel (the fused step; the E
pass when the two-pass kernels run) timed live with CUDA events against the measured
HBM copy bandwidth, on the bytes it moves; cpu_baseline = the CPU
oracle (scipy sparse operator, the reference's algorithm) on a bounded slab of the
same workload.
"""

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mcell-updates/s & % HBM roofline; served solves/h, p99 at WP err≤1e-4 vs FP64"
MM = 1e-3

# algorithmic bytes per cell and launch (FP32 words x 4 B): H pass reads E, H, ch and
# writes H (12 words); E pass reads H, E, ce, cl and writes E (15 words, lossy grid).
# A full step of one cell: 12 E/H words + 3 ch + 3 ce + 3 cl = 21 words = 84 B (the
# fused-step figure; the two-pass step moves 27 words).
BYTES_H, BYTES_E, BYTES_STEP_MODEL = 48, 60, 84
BYTES_FIELDS = 48  # E and H, 6 FP32 words, each read and written once


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ----------------------------------------------------------------------------- workload
class Pillbox:
    nx, ny, nz = 512, 512, 1024
    half_xy = 55 * MM
    zmax = 200 * MM
    R, L, rp = 50 * MM, 100 * MM, 10 * MM
    sigma = 5.8e7
    n_pml = 16
    sigmaz = 5 * MM
    wakelength = 0.3
    cfln = 0.5

    def __init__(self, nx=None, ny=None, nz=None):
        if nx:
            self.nx, self.ny, self.nz = nx, ny, nz

    def axes(self):
        return (np.linspace(-self.half_xy, self.half_xy, self.nx + 1),
                np.linspace(-self.half_xy, self.half_xy, self.ny + 1),
                np.linspace(-self.zmax, self.zmax, self.nz + 1))

    def walls_mask(self, device=None, zslab=None):
        """Wall cells (C order over (nx, ny, nz)) at cell centres, as a torch bool tensor
        on `device` or a numpy array when device is None."""
        x, y, z = self.axes()
        xc, yc, zc = x[:-1] + np.diff(x) / 2, y[:-1] + np.diff(y) / 2, z[:-1] + np.diff(z) / 2
        if zslab is not None:
            zc = zc[zslab]
        if device is None:
            r2 = xc[:, None, None] ** 2 + yc[None, :, None] ** 2
            zz = zc[None, None, :]
            vac = ((r2 <= self.R ** 2) & (np.abs(zz) <= self.L / 2)) | (r2 <= self.rp ** 2)
            return ~vac
        import torch
        X = torch.as_tensor(xc, device=device)[:, None, None]
        Y = torch.as_tensor(yc, device=device)[None, :, None]
        Z = torch.as_tensor(zc, device=device)[None, None, :]
        r2 = X ** 2 + Y ** 2
        vac = ((r2 <= self.R ** 2) & (Z.abs() <= self.L / 2)) | (r2 <= self.rp ** 2)
        return ~vac

    def build(self, wg, mask, dtype=np.float32, results=None, dt=None):
        x, y, z = self.axes()
        grid = wg.GridFIT3D(x=x, y=y, z=z, stl_solids={"walls": mask},
                            stl_materials={"walls": [1.0, 1.0, self.sigma]}, verbose=0)
        wake = wg.WakeSolver(wakelength=self.wakelength, q=1e-9, sigmaz=self.sigmaz, beta=1.0, save=False,
                             verbose=0, results_folder=results or tempfile.mkdtemp())
        solver = wg.SolverFIT3D(grid, wake, cfln=self.cfln, dt=dt, bc_low=["pec", "pec", "pml"],
                                bc_high=["pec", "pec", "pml"], use_stl=True, bg=[1.0, 1.0], dtype=dtype,
                                n_pml=self.n_pml, verbose=0)
        return grid, wake, solver


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    def __init__(self, out_path):
        self.path = out_path
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self, device_index=0):
        try:
            rows = [ln.split(",") for ln in open(self.path).read().strip().splitlines()]
        except Exception:
            return None
        rows = [[c.strip() for c in r] for r in rows if len(r) >= 9 and r[0].strip() == str(device_index)]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows]
        smax = max(float(r[2]) for r in rows)
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for nm, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(rows), "power_w_max": max(float(r[3]) for r in rows if r[3] not in ("", "[N/A]"))}


# ----------------------------------------------------------------------------- CPU side
def _cpu_worker(nz_slab, steps, budget_s, barrier, out):
    """One host process stepping the oracle on its own slab (spawned: no CUDA state)."""
    sys.path.insert(0, ROOT)
    rate, _, _ = cpu_sample_rate(nz_slab, steps, budget_s, barrier=barrier)
    out.put(rate)


def cpu_sample_parallel(workers=None, nz_slab=16, steps=20, budget_s=20.0):
    """The CPU oracle on all host cores: one single-threaded scipy process per core, each
    on its own slab of the pillbox grid, stepping at the same time (a barrier after the
    set-up); the rates add.  Returns (Mcell-updates/s, description, processes)."""
    import multiprocessing as mp
    workers = workers or min(os.cpu_count() or 1, 16)
    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(workers)
    out = ctx.Queue()
    procs = [ctx.Process(target=_cpu_worker, args=(nz_slab, steps, budget_s, barrier, out)) for _ in range(workers)]
    for p in procs:
        p.start()
    rates = [out.get() for _ in procs]
    for p in procs:
        p.join()
    P = Pillbox()
    return sum(rates), (f"oracle one_step (scipy CSR, FP32; the reference's algorithm) in {workers} concurrent "
                        f"single-threaded processes, each on its own {P.nx}x{P.ny}x{nz_slab} slab of the pillbox "
                        f"grid, up to {steps} steps or {budget_s:.0f} s after 1 warm-up step; rates summed"), workers


def cpu_sample_rate(nz_slab=16, steps=20, budget_s=25.0, barrier=None):
    """The CPU oracle (scipy CSR leapfrog, one core) on a z slab of the pillbox grid:
    returns (Mcell-updates/s, description)."""
    from oracle import fit_oracle as O
    P = Pillbox()
    x, y, z = P.axes()
    k0 = P.nz // 2 - nz_slab // 2
    zs = z[k0:k0 + nz_slab + 1]
    g = O.OracleGrid(x, y, zs)
    mask = P.walls_mask(zslab=slice(k0, k0 + nz_slab))
    s = O.OracleSolver(g, ["pec", "pec", "pml"], ["pec", "pec", "pml"], solids=[(mask, [1.0, 1.0, P.sigma])],
                       bg=[1.0, 1.0], cfln=P.cfln, dtype=np.float32, n_pml=2)
    rng = np.random.default_rng(0)
    s.E[:] = rng.standard_normal(s.E.size).astype(np.float32)
    s.one_step()
    if barrier is not None:
        barrier.wait()
    done = 0
    t0 = time.perf_counter()
    while done < steps and (time.perf_counter() - t0) < budget_s:
        s.one_step()
        done += 1
    dt = time.perf_counter() - t0
    rate = g.N * done / dt / 1e6
    return rate, f"oracle one_step (scipy CSR, FP32) on a {P.nx}x{P.ny}x{nz_slab} slab of the pillbox grid, " \
                 f"{done} steps after 1 warm-up step", 1


# ----------------------------------------------------------------------------- runs
def run_cpu_workloads(args):
    """The CPU oracle (scipy CSR leapfrog, the reference's algorithm, one thread) on the
    60x60x120 cavity, 128x128x256 lossy cavity and 256^3 sphere grids in FP64 and FP32: Mcell-updates/s over --cpu-steps steps after
    one warm-up step (random fields), and the 60x60x120 cavity's time-to-impedance (its whole
    FP64 wakesolve, set-up included).  Prints one JSON line."""
    for p in (os.path.join(ROOT, "tests"), os.path.join(ROOT, "tests", "golden")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import cases as C
    from oracle_runner import oracle_solver, run_oracle_case
    rates = {}
    for name in ("cavity_60x60x120", "lossy_cavity_128x128x256", "sphere_packet_256"):
        for dt in ("float64", "float32"):
            t0 = time.perf_counter()
            s = oracle_solver(dict(C.WORKLOADS[name], dtype=dt))
            setup = time.perf_counter() - t0
            rng = np.random.default_rng(0)
            s.E[:] = rng.standard_normal(s.E.size).astype(s.E.dtype)
            s.one_step()
            t0 = time.perf_counter()
            for _ in range(args.cpu_steps):
                s.one_step()
            sec = time.perf_counter() - t0
            rates[f"{name}_{dt}"] = {"cells": int(s.N), "steps": args.cpu_steps, "seconds": sec,
                                     "mcell_updates_per_s": s.N * args.cpu_steps / sec / 1e6,
                                     "operator_setup_s": setup}
            del s
    t0 = time.perf_counter()
    r = run_oracle_case("cavity_60x60x120", case=C.WORKLOADS["cavity_60x60x120"])
    tti = time.perf_counter() - t0
    print(json.dumps({"mode": "cpu_workloads", "impl": "oracle (scipy CSR, one thread)", "threads": 1,
                      "host_cpus": os.cpu_count(), "rates": rates,
                      "cavity_60x60x120_time_to_impedance": {"seconds": tti, "steps": int(r["Nt"]),
                                                    "what": "FP64 wakesolve of the 60x60x120 cavity through the oracle, "
                                                            "grid and operator set-up included"}}), flush=True)


def run_reference(args, rank, world):
    if rank != 0:
        return
    rate, sample, cores = cpu_sample_parallel(steps=max(args.steps, 1))
    line = {"impl": "reference", "metric": METRIC, "value": rate, "unit": "Mcell-updates/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (analytic pillbox geometry)",
            "config": {"workload": "pillbox 512x512x1024 FP32 (bounded z-slab sample on the host)"},
            "cpu_baseline": {"value": rate, "unit": "Mcell-updates/s", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": rate, "unit": "Mcell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def replica_max_ms(ms, device, world):
    """The timed region's milliseconds, max over the ranks (a barrier first): the
    replicas' job time."""
    import torch
    t = torch.tensor([float(ms)], device=device, dtype=torch.float64)
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_value(cells, steps, world, ms):
    """Whole-job Mcell-updates/s: every rank steps its own full grid (weak scaling)."""
    return cells * steps * world / (ms / 1e3) / 1e6


def run_ours(args, rank, world):
    import torch
    import wakis_gb300 as wg
    from wakis_gb300 import _native as nat

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    P = Pillbox(*args.grid) if args.grid else Pillbox()
    N = P.nx * P.ny * P.nz
    mask = P.walls_mask(device=dev)
    grid, wake, s = P.build(wg, mask)
    s.kernels = args.variant
    s.coefficient_codes = not args.dense
    tuned = None
    if s.kernels == "fused":
        if args.fused_shape:
            s._ctx.call("fit_set_fused_shape", *args.fused_shape)
            s._sync_coeffs()
            s._ensure_codes()
            s.fused_staging = args.staging
            tuned = {tuple(args.fused_shape) + (args.staging, 1 if args.staging else 0): float("nan")}
        else:
            tuned = s.tune_fused()
    del mask
    beam, Nt = s._wake_prepare(wake, P.wakelength, "both")
    vt = s._wake_device_setup(beam, Nt)
    n = s._wake_first_step(beam)
    K, W = args.steps, args.warmup
    if n + W + K > Nt:
        raise SystemExit(f"steps {W}+{K} exceed the run length {Nt}")
    s._device_steps(n, W)
    n += W
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    # the nvidia-smi samples of the timed region (summarised into the line's "clocks")
    clk_dir = os.environ.get("WAKIS_BENCH_CLOCKS_DIR") or tempfile.gettempdir()
    clk_path = os.path.join(clk_dir, f"clocks_rank{rank}.csv")
    os.makedirs(os.path.dirname(clk_path), exist_ok=True)
    launches0 = nat.launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(clk_path) as clk:
        time.sleep(0.3)
        ev0.record()
        s._device_steps(n, K)
        ev1.record()
        torch.cuda.synchronize()
    launches = nat.launch_count() - launches0
    ms = replica_max_ms(ev0.elapsed_time(ev1), dev, world)
    n += K
    value = replica_value(N, K, world, ms)
    # live per-kernel timing (same context, same stream)
    kt = np.zeros(2)
    s._ctx.call("fit_time_kernels", 10, nat.dptr(kt))
    peak, src = peaks()
    coded = s.coefficient_code_count > 0
    # two-pass passes: dense H 48 B / E 60 B per cell; coded both 38 B (fields + a code)
    bytes_e, bytes_h = (BYTES_FIELDS // 2 + 12 + 2, BYTES_FIELDS // 2 + 12 + 2) if coded else (BYTES_E, BYTES_H)
    ach_e = bytes_e * N / (kt[1] / 1e3) / 1e9
    ach_h = bytes_h * N / (kt[0] / 1e3) / 1e9
    ach_step = BYTES_STEP_MODEL * N / (ms / K / 1e3) / 1e9
    traffic = profile_traffic("epass_coded_pillbox_ncu.md" if coded else "epass_pillbox_ncu.md")
    fused = None
    if s.kernels == "fused":
        kf = np.zeros(1)
        s._ctx.call("fit_time_fused", 10, nat.dptr(kf))
        # coded: E and H read and written once (48 B) + a 2-byte code per cell; the code
        # table (coefficient_code_count x 48 B) stays in L1/L2
        bytes_cell = BYTES_FIELDS + 2 if coded else BYTES_STEP_MODEL
        ach_f = bytes_cell * N / (kf[0] / 1e3) / 1e9
        fused = {"bound": "hbm", "kernel": "k_step_fused (whole step, lossy, FP32%s)" % (", coded coefficients"
                                                                                         if coded else ""),
                 "achieved": ach_f, "peak": peak, "unit": "GB/s", "frac": ach_f / peak,
                 "traffic": profile_traffic("fused_coded_pillbox_ncu.md" if coded else "fused_pillbox_ncu.md"),
                 "algorithmic_bytes_per_launch": bytes_cell * N, "ms_per_launch": kf[0],
                 "peak_source": f"{src} HBM copy bandwidth (MEASURED_PEAKS.json hbm_gbs)"}
        fused["traffic_source"] = ("profiles/%s: ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch on "
                                   "the 256x256x512 grid, scaled by the cell count (x8)"
                                   % ("fused_coded_pillbox_ncu.md" if coded else "fused_pillbox_ncu.md"))
        if coded:
            ach_model = BYTES_STEP_MODEL * N / (kf[0] / 1e3) / 1e9
            fused["coefficient_codes"] = s.coefficient_code_count
            fused["model_84B"] = {"achieved": ach_model, "frac": ach_model / peak,
                                  "note": "the 84 B/cell-update model (dense ch, ce, cl) at the coded step's speed; "
                                          "above 1 because the coded step moves 50 B per cell, not 84"}
    out = {"metric": METRIC, "value": value, "unit": "Mcell-updates/s", "n_gpus": world, "steps": K, "warmup": W,
           "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (analytic pillbox geometry, Gaussian beam)",
           "config": {"workload": f"pillbox {P.nx}x{P.ny}x{P.nz} FP32, sigma=5.8e7 walls (relaxation form), "
                                  f"16-cell z PML, beam sigma_z=5 mm, 3x3 wake taps",
                      "cells": N, "run_steps": Nt, "cfln": P.cfln, "dt": float(s.dt),
                      "l2": "no flush: inputs (14 GB per step coded, 22 GB dense) far larger than the 129 MB L2",
                      "parallelism": "replicas" if world > 1 else "single GPU"},
           "roofline": {"bound": "hbm", "kernel": "k_epass%s (E pass, lossy, FP32)" % ("_coded" if coded else ""),
                        "achieved": ach_e, "peak": peak, "unit": "GB/s", "frac": ach_e / peak, "traffic": traffic,
                        "algorithmic_bytes_per_launch": bytes_e * N, "ms_per_launch": kt[1],
                        "peak_source": f"{src} HBM copy bandwidth (MEASURED_PEAKS.json hbm_gbs)"},
           "roofline_hpass": {"achieved": ach_h, "frac": ach_h / peak, "ms_per_launch": kt[0],
                              "algorithmic_bytes_per_launch": bytes_h * N},
           "step_roofline": {"model_bytes_per_cell": BYTES_STEP_MODEL, "achieved": ach_step, "frac": ach_step / peak,
                             "note": "84 B/cell-update = fused-step algorithmic bytes; the two-pass step moves "
                                     "108 B/cell"},
           "gpu_launches": int(launches)}
    out["roofline"]["traffic_source"] = ("profiles/%s: ncu dram bytes of one launch on the 256x256x512 grid, "
                                         "scaled by the cell count (x8)"
                                         % ("epass_coded_pillbox_ncu.md" if coded else "epass_pillbox_ncu.md"))
    if fused is not None and coded and not args.no_dense_roofline:
        # the dense fused step on the same grid (84 B per cell-update: ch, ce, cl read per
        # cell), the step a grid with more than 65535 distinct coefficient triples runs
        s.coefficient_codes = False
        s._ensure_codes()
        s._ctx.call("fit_set_fused_staging", 0, 0)
        kd = np.zeros(2)
        dense_ms = {}
        for shape in ((4, 4, 64, 3), (4, 4, 64, 4), (4, 8, 64, 2), (4, 4, 32, 3)):
            s._ctx.call("fit_set_fused_shape", *shape)
            s._ctx.call("fit_time_fused", 10, nat.dptr(kd))
            dense_ms[shape] = float(kd[0])
        shape = min(dense_ms, key=dense_ms.get)
        ach_d = BYTES_STEP_MODEL * N / (dense_ms[shape] / 1e3) / 1e9
        out["roofline_dense"] = {"bound": "hbm", "kernel": "k_step_fused (whole step, lossy, FP32, dense coefficients)",
                                 "achieved": ach_d, "peak": peak, "unit": "GB/s", "frac": ach_d / peak,
                                 "algorithmic_bytes_per_launch": BYTES_STEP_MODEL * N, "ms_per_launch": dense_ms[shape],
                                 "shape": {"vec": shape[0], "rows": shape[1], "zseg": shape[2], "ctas": shape[3]},
                                 "ms_by_shape": {"v%dr%dz%dc%d" % k: t for k, t in dense_ms.items()},
                                 "traffic": profile_traffic("fused_pillbox_ncu.md"),
                                 "traffic_source": "profiles/fused_pillbox_ncu.md (ncu, 256x256x512 grid, scaled x8)",
                                 "note": "the fused step of a grid whose coefficients do not compress (more than "
                                         "65535 distinct triples, e.g. graded spacing): 84 B per cell-update"}
    if fused is not None:
        out["roofline_two_pass_e"] = out["roofline"]
        out["roofline"] = fused
        shapes = {k: t for k, t in tuned.items() if k != "two-pass"}
        best = min(shapes, key=lambda t: shapes[t] if shapes[t] == shapes[t] else 0.0)
        out["fused_autotune"] = {"best": list(best),
                                 "ms_per_step": {f"v{v}r{r}z{z}c{m}s{st}a{a}": t
                                                 for (v, r, z, m, st, a), t in sorted(shapes.items())},
                                 "two_pass_ms_per_step": tuned.get("two-pass")}
        out["config"]["kernels"] = "fused single-pass step (ping-pong field buffers)"
        if len(best) > 4 and best[4]:
            out["roofline"]["kernel"] = out["roofline"]["kernel"].replace("k_step_fused", "k_step_tma (TMA plane rings)")
            out["config"]["kernels"] += ", old fields fed by TMA plane rings"
    else:
        out["config"]["kernels"] = f"{s.kernels} H and E pass kernels"
    csum = clk.summary(dev.index)
    if csum is not None:
        out["clocks"] = csum
    del s, grid, wake
    import gc
    gc.collect()
    torch.cuda.empty_cache()
    if not args.no_e2e:
        out["e2e"] = e2e(wg, torch, dev, P, args.variant)
    if rank == 0 and world == 1 and not args.no_serve:
        out["serving"] = serving_summary(args, peak)
    if rank == 0 and not args.no_cpu:
        rate, sample, cores = cpu_sample_parallel()
        out["cpu_baseline"] = {"value": rate, "unit": "Mcell-updates/s", "cores": cores, "kind": "port",
                               "sample": sample}
    if rank == 0:
        print(json.dumps(out), flush=True)


def serving_summary(args, peak):
    """The served path, measured in the default run on one GPU (the second half of the
    metric: served solves/h and p99): the 64-request cavity sweep (cube 20-60 mm, n 48-160, default_rng(seed=3)),
    arriving as a Poisson stream at which the 4 GB memory budget binds, served in FP32 by
    the pool with continuous batching (two-pass kernel variants chosen by the autotuner on
    calibration grids); the pool's throughput with every request resident, over the first
    0.1 m of wake (a per-step rate, which the wake length does not change), against the
    measured HBM bandwidth; and the plain FP64 path one request at a time on a seeded
    subsample, which gives the FP64 solves/h and each subsampled request's WP / Z error of
    the served FP32 result (the FP64 runs take the FP32 time step)."""
    import gc
    import torch
    from wakis_gb300 import serving as S
    from wakis_gb300 import _native as nat

    def free():
        gc.collect()
        torch.cuda.empty_cache()

    t_all = time.perf_counter()
    budget = int(args.serve_budget_gb * 1e9)
    base = S.cavity_sweep_requests(args.serve_count, seed=3)
    rate = S.poisson_rate_for(base, budget, args.serve_ref_rate * 1e9, load=args.serve_load)
    reqs = S.cavity_sweep_requests(args.serve_count, seed=3, rate_hz=rate)
    out = {"workload": f"{len(reqs)} cavity wake solves (cube 20-60 mm, pipe 3-8 mm, n 48-160, z 2n, sigma_z 5-15 mm, "
                       f"PEC or sigma 1e3-1e6 S/m, wake 1 m), default_rng(seed=3)",
           "budget_bytes": budget, "arrival_rate_hz": rate, "chunk_steps": args.serve_chunk,
           "arrivals": f"Poisson, {args.serve_load}x the service rate of {args.serve_ref_rate} G cell-updates/s"}
    warm = [S.CavityRequest(tag=1000 + i, side=20e-3, rp=4e-3, n=16 + 2 * i, sigmaz=6e-3, sigma=1e4 * i,
                            wakelength=0.05) for i in range(2)]
    loop = S.ServingLoop(budget, chunk_steps=args.serve_chunk, keep_results=False)
    loop.run(warm)
    loop.close()
    t0 = time.perf_counter()
    tpool = nat.Pool(32 << 30, chunk_steps=args.serve_chunk)
    tuned = S.autotune(tpool)
    tpool.close()
    free()
    variants = {vec: r["choice"] for vec, r in tuned.items()}
    out["autotune"] = {"seconds": time.perf_counter() - t0, "choice": {str(v): m for v, m in variants.items()}}
    # FP32 served, Poisson arrivals, memory admission
    loop = S.ServingLoop(budget, chunk_steps=args.serve_chunk, variants=variants)
    recs, summ = loop.run(reqs)
    res32 = loop.results
    loop.close()
    free()
    out["solves_per_hour"] = summ["solves_per_hour"]
    out["tti_p50_s"], out["tti_p99_s"] = summ["tti_p50_s"], summ["tti_p99_s"]
    out["makespan_s"] = summ["makespan_s"]
    out["mcell_updates_per_s"] = summ["mcell_updates_per_s"]
    out["solves"], out["failed"] = summ["solves"], summ["failed"]
    out["max_resident"] = summ["pool"]["max_active"]
    # every request resident: the pool's per-step throughput against the bytes its coded
    # two-pass kernels move (76 B per cell-update: E and H read and written once per pass
    # and a 2-byte code per pass) and against the 72 / 84 B per cell-update model
    short = S.cavity_sweep_requests(args.serve_count, seed=3, wakelength=0.1)
    pool = nat.Pool(sum(S.footprint_bytes(r) for r in short) + (1 << 30), chunk_steps=args.serve_chunk)
    for vec, m in variants.items():
        pool.tune(vec, m)
    cu, busy, jobs = S.run_resident(pool, short, kernels="direct")
    st = pool.stats()
    pool.close()
    coded = all(j.solver.coefficient_code_count > 0 for j in jobs)
    moved = sum((76 if j.solver.coefficient_code_count > 0 else (108 if j.req.lossy else 96)) * j.req.cells
                * (j.Nt - j.first) for j in jobs)
    model = sum((84 if j.req.lossy else 72) * j.req.cells * (j.Nt - j.first) for j in jobs)
    for j in jobs:
        j.close()
    del jobs
    free()
    out["all_resident"] = {"requests": len(short), "wake_m": 0.1, "seconds": busy, "mcell_updates_per_s": cu / busy / 1e6,
                           "hbm_gbs": moved / busy / 1e9, "hbm_frac": moved / busy / 1e9 / peak,
                           "hbm_frac_model": model / busy / 1e9 / peak, "coded": coded, "chunks": st["chunks"],
                           "bytes": "hbm_frac on the 76 B per cell-update the coded two-pass kernels move; "
                                    "hbm_frac_model on the 72 B (PEC) / 84 B (lossy) model"}
    # plain FP64 one at a time on a subsample: solves/h and the FP32 results' errors
    if args.serve_fp64_sample <= 0:
        out["seconds"] = time.perf_counter() - t_all
        return out
    rng = np.random.default_rng(5)
    sub = sorted(rng.choice(len(reqs), size=min(args.serve_fp64_sample, len(reqs)), replace=False).tolist())
    res64 = {}
    t0 = time.perf_counter()
    for i in sub:
        r = reqs[i]
        res64[r.tag] = S.solve_alone(r, np.float64, dt=S.cfl_dt(r, np.float32), kernels="auto")
        torch.cuda.synchronize()
        free()
    sec64 = time.perf_counter() - t0
    frac_work = sum(reqs[i].cells * S._steps_estimate(reqs[i]) for i in sub) / sum(
        r.cells * S._steps_estimate(r) for r in reqs)
    fp64_sph = len(reqs) * 3600.0 * frac_work / sec64  # the whole sweep at the subsample's rate
    wp = {t: _rel(res32[t]["WP"], res64[t]["WP"]) for t in res64 if t in res32}
    zz = {t: _rel(res32[t]["Z"], res64[t]["Z"]) for t in res64 if t in res32}
    out["plain_fp64_one_at_a_time"] = {
        "sample": f"{len(sub)} of {len(reqs)} requests (default_rng(5)), run back to back; solves/h scaled by their "
                  f"share of the sweep's cell-updates ({frac_work:.3f})",
        "seconds": sec64, "solves_per_hour": fp64_sph}
    out["speedup_solves_per_hour_vs_fp64"] = summ["solves_per_hour"] / fp64_sph
    out["accuracy_vs_fp64"] = {"WP_rel_l2_max": max(wp.values()), "WP_rel_l2_median": float(np.median(list(wp.values()))),
                               "Z_rel_l2_max": max(zz.values()), "requests": len(wp),
                               "requests_above_1e-4": int(sum(e > 1e-4 for e in wp.values()))}
    out["seconds"] = time.perf_counter() - t_all
    return out


def e2e(wg, torch, dev, P, kernels="direct"):
    """Complete wakesolve through the public API: host numpy geometry -> GridFIT3D ->
    SolverFIT3D -> wakesolve -> WP / WPx / WPy / Z / Zx / Zy back on the host."""
    torch.cuda.synchronize()
    mask = P.walls_mask()  # host, numpy
    h2d = mask.nbytes
    t0 = time.perf_counter()
    grid, wake, s = P.build(wg, mask)
    s.kernels = kernels
    s.wakesolve(wakelength=P.wakelength)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    Nt = s.Nt
    d2h = sum(np.asarray(a).nbytes for a in (wake.WP_3d, wake.WPx, wake.WPy, wake.Z, wake.Zx, wake.Zy))
    N = P.nx * P.ny * P.nz
    return {"value": N * Nt / dt / 1e6, "unit": "Mcell-updates/s", "h2d_bytes_per_step": h2d / Nt,
            "d2h_bytes_per_step": d2h / Nt, "steps": Nt, "seconds": dt,
            "what": "GridFIT3D + SolverFIT3D setup from a host mask, wakesolve(0.3 m), WakeSolver results on host"}


def _rel(a, b, ref=None):
    a, b = np.asarray(a, dtype=np.complex128), np.asarray(b, dtype=np.complex128)
    den = np.linalg.norm(b)
    if ref is not None:
        den = max(den, 1e-3 * np.linalg.norm(np.asarray(ref, dtype=np.complex128)))
    return float(np.linalg.norm(a - b) / den) if den > 0 else float(np.linalg.norm(a - b))


def run_accuracy(args):
    """FP32 runs against the FP64 CUDA path (validated against the CPU oracle at 1e-10):
    the lossy 128x128x256 cavity (both beam runs: fields, WP, WPx, WPy, Z, Zx, Zy), the
    256^3 sphere (64 probes of Ez over 2000 steps) and, with --accuracy-pillbox, the
    512x512x1024 pillbox (WP over the first 0.3 m).

    An FP32 solver rounds dt to float32, as the reference does.  The main comparison
    ("same_dt") runs FP64 at that rounded dt, so it isolates field precision.  The second
    ("cfl_dt") runs FP64 at its own CFL step.  Its gap adds the post-processor's
    sensitivity to dt: the wake time index int(.../dt) flips for some (s, z) pairs.
    """
    import gc
    import torch
    import wakis_gb300 as wg
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import cases as CS
    from product_runner import make_grid, make_solver
    out = {}
    tmp = tempfile.mkdtemp()

    def free():
        gc.collect()
        torch.cuda.empty_cache()

    def wake_run(case, dtype, dt=None):
        grid = make_grid(wg, case)
        wake = wg.WakeSolver(wakelength=case["wakelength"], save=False, verbose=0, results_folder=tmp,
                             **case["wake"])
        s = make_solver(wg, case, grid, wake, dtype, dt)
        t0 = time.perf_counter()
        s.wakesolve(wakelength=case["wakelength"])
        torch.cuda.synchronize()
        r = dict(sec=time.perf_counter() - t0, Nt=s.Nt, dt=float(s.dt), s=wake.s, WP=wake.WP, WPx=wake.WPx,
                 WPy=wake.WPy, Z=wake.Z, Zx=wake.Zx, Zy=wake.Zy, E=s.E.numpy(), H=s.H.numpy())
        del s, grid, wake
        free()
        return r

    def wake_err(a, b):
        n = min(len(a["WP"]), len(b["WP"]))
        m = min(len(a["Z"]), len(b["Z"]))
        return {"WP": _rel(a["WP"][:n], b["WP"][:n]), "WPx": _rel(a["WPx"][:n], b["WPx"][:n], b["WP"][:n]),
                "WPy": _rel(a["WPy"][:n], b["WPy"][:n], b["WP"][:n]), "Z": _rel(a["Z"][:m], b["Z"][:m]),
                "Zx": _rel(a["Zx"][:m], b["Zx"][:m], b["Z"][:m]), "Zy": _rel(a["Zy"][:m], b["Zy"][:m], b["Z"][:m]),
                "E": _rel(a["E"], b["E"]), "H": _rel(a["H"], b["H"]), "Nt": [a["Nt"], b["Nt"]]}

    for name in ("lossy_cavity_128x128x256", "lossy_cavity_128x128x256_offset"):
        case = CS.WORKLOADS[name]
        a = wake_run(case, np.float32)
        b = wake_run(case, np.float64, a["dt"])
        c = wake_run(case, np.float64)
        out[name] = {"same_dt": wake_err(a, b), "cfl_dt": wake_err(a, c), "dt_fp32": a["dt"], "dt_fp64": c["dt"],
                     "seconds_fp32": a["sec"], "seconds_fp64": b["sec"]}
    # the sphere and wave packet: probes
    case = CS.WORKLOADS["sphere_packet_256"]
    P = CS.probe_points(case)
    probes = {}
    dt32 = None
    for key, dtype in (("fp32", np.float32), ("fp64", np.float64)):
        grid = make_grid(wg, case)
        s = make_solver(wg, case, grid, dtype=dtype, dt=dt32)
        dt32 = float(s.dt)
        sc = case["source"]
        src = wg.sources.WavePacket(zs=sc["zs"], sigmaz=sc["sigmaz"], sigmaxy=sc["sigmaxy"],
                                    wavelength=sc["wavelength"], amplitude=sc["amplitude"])
        flat = torch.as_tensor(2 * s.N + P[:, 0] + s.Nx * P[:, 1] + s.Nx * s.Ny * P[:, 2], device=s.E.array.device)
        rec = []
        t0 = time.perf_counter()
        s.emsolve(case["Nt"], source=src, callback=lambda sv, t: rec.append(sv.E.array[flat].double()))
        torch.cuda.synchronize()
        probes[key] = (torch.stack(rec).cpu().numpy(), time.perf_counter() - t0)
        del s, grid
        free()
    a, b = probes["fp32"][0], probes["fp64"][0]
    out["sphere_packet_256"] = {"probe_Ez_rel_l2": _rel(a, b), "probe_Ez_max_abs_over_max": float(np.abs(a - b).max()
                                                                                        / np.abs(b).max()),
                      "steps": case["Nt"], "probes": int(len(P)), "dt": "FP64 run at the FP32 run's dt",
                      "seconds_fp32": probes["fp32"][1], "seconds_fp64": probes["fp64"][1]}
    if args.accuracy_pillbox:
        P4 = Pillbox()
        res = {}
        dt32 = None
        for key, dtype in (("fp32", np.float32), ("fp64", np.float64)):
            mask = P4.walls_mask(device=torch.device("cuda", 0))
            grid, wake, s = P4.build(wg, mask, dtype=dtype, dt=dt32)
            dt32 = float(s.dt)
            del mask
            t0 = time.perf_counter()
            s.wakesolve(wakelength=P4.wakelength)
            torch.cuda.synchronize()
            res[key] = dict(sec=time.perf_counter() - t0, s=wake.s, WP=wake.WP, Z=wake.Z, Nt=s.Nt)
            del s, grid, wake
            free()
        a, b = res["fp32"], res["fp64"]
        out["pillbox_512x512x1024"] = {"WP_first_0.3m": _rel(a["WP"], b["WP"]), "Z": _rel(a["Z"], b["Z"]),
                          "Nt": [a["Nt"], b["Nt"]], "dt": "FP64 run at the FP32 run's dt",
                          "seconds_fp32": a["sec"], "seconds_fp64": b["sec"]}
    print(json.dumps({"accuracy": out}), flush=True)


def run_serve(args):
    """Served wake solves (the 64-request cavity sweep): FP32 continuous batching through
    the pool against the plain FP64 path one request at a time, on the same requests and
    Poisson arrivals; per-request WP / Z errors of the served FP32 results against the
    FP64 ones (run at the FP32 time step); the pool's throughput with every request
    resident; and the CPU oracle's per-core rate extrapolated to the same requests."""
    import gc
    import torch
    import wakis_gb300 as wg  # noqa: F401  (builds / loads the library)
    from wakis_gb300 import serving as S
    from wakis_gb300 import _native as nat

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    peak, src = peaks()
    budget = int(args.serve_budget_gb * 1e9)
    base = S.cavity_sweep_requests(args.serve_count, seed=3)
    rate = S.poisson_rate_for(base, budget, args.serve_ref_rate * 1e9, load=args.serve_load)
    reqs = S.cavity_sweep_requests(args.serve_count, seed=3, rate_hz=rate)
    work_bytes = {r.tag: (84 if r.lossy else 72) for r in reqs}

    def model_bytes(recs):
        return sum(work_bytes[r["tag"]] * r["cells"] * r["steps"] for r in recs)

    # warm-up: library, graphs and allocator on two tiny requests
    warm = [S.CavityRequest(tag=1000 + i, side=20e-3, rp=4e-3, n=16 + 2 * i, sigmaz=6e-3, sigma=1e4 * i,
                            wakelength=0.05) for i in range(2)]
    loop = S.ServingLoop(budget, chunk_steps=args.serve_chunk, keep_results=False)
    loop.run(warm)
    loop.close()

    out = {"metric": METRIC, "impl": "ours", "mode": "serve", "n_gpus": 1, "dtype": "f32 fields, f64 wake sums and DFT",
           "data": "synthetic (seeded cavity requests, analytic geometry)",
           "config": {"workload": f"{len(reqs)} cavity wake solves (cube 20-60 mm, pipe 3-8 mm, n 48-160 cells, "
                                  f"z 2n, sigma_z 5-15 mm, PEC or sigma 1e3-1e6 S/m, wake 1 m), "
                                  f"default_rng(seed=3)",
                      "budget_bytes": budget, "arrival_rate_hz": rate,
                      "arrivals": f"Poisson, {args.serve_load}x the service rate of {args.serve_ref_rate} G "
                                  f"cell-updates/s (the memory budget binds)",
                      "chunk_steps": args.serve_chunk,
                      "total_cell_updates": int(sum(r.cells * S._steps_estimate(r) for r in reqs))}}

    # autotuner: pass-kernel variant per vector-width class, timed on calibration grids
    t_tune = time.perf_counter()
    tpool = nat.Pool(32 << 30, chunk_steps=args.serve_chunk)
    tuned = S.autotune(tpool)
    tpool.close()
    gc.collect()
    torch.cuda.empty_cache()
    variants = {vec: r["choice"] for vec, r in tuned.items()}
    out["autotune"] = {"seconds": time.perf_counter() - t_tune,
                       "classes": {str(v): {"choice": r["choice"],
                                            "G_cell_updates_per_s": {str(m): x / 1e9 for m, x in r["rates"].items()}}
                                   for v, r in tuned.items()}}

    # FP32 served
    loop = S.ServingLoop(budget, chunk_steps=args.serve_chunk, variants=variants)
    recs, summ = loop.run(reqs)
    res32 = loop.results
    loop.close()
    gc.collect()
    torch.cuda.empty_cache()
    mb = model_bytes(recs)
    summ["hbm_gbs_model"] = mb / summ["makespan_s"] / 1e9
    summ["hbm_frac_model"] = summ["hbm_gbs_model"] / peak
    busy = summ["pool"]["busy_ms"] / 1e3
    summ["hbm_gbs_model_while_busy"] = mb / busy / 1e9 if busy > 0 else None
    out["served_fp32"] = summ
    out["value"] = summ["solves_per_hour"]
    out["unit"] = "solves/h"
    out["higher_is_better"] = True
    out["tti_p50_s"], out["tti_p99_s"] = summ["tti_p50_s"], summ["tti_p99_s"]

    # the pool with every request resident (kernel throughput of the batched passes)
    if not args.serve_no_saturated:
        jobs = [S.ServedSolve(r) for r in reqs]
        pool = nat.Pool(sum(S.footprint_bytes(r) for r in reqs) + (1 << 30), chunk_steps=args.serve_chunk)
        for vec, m in variants.items():
            pool.tune(vec, m)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for j in jobs:
            j.submit(pool)
        done = []
        while len(done) < len(jobs):
            done += pool.poll(wait_ms=100)
        el = time.perf_counter() - t0
        st = pool.stats()
        pool.close()
        cu = sum(j.req.cells * (j.Nt - j.first) for j in jobs)
        mbs = sum(work_bytes[j.req.tag] * j.req.cells * (j.Nt - j.first) for j in jobs)
        # bytes the pool's two-pass kernels move per cell-update: coded 76 B (E and H read
        # and written once per pass, a 2-byte code per pass), dense 96 B (PEC) / 108 B (lossy)
        coded = [j.solver.coefficient_code_count > 0 for j in jobs]
        two_pass = sum((76 if cd else (108 if j.req.lossy else 96)) * j.req.cells * (j.Nt - j.first)
                       for j, cd in zip(jobs, coded))
        out["pool_all_resident"] = {"requests": len(jobs), "seconds": el, "mcell_updates_per_s": cu / el / 1e6,
                                    "hbm_gbs_model": mbs / el / 1e9, "hbm_frac_model": mbs / el / 1e9 / peak,
                                    "hbm_gbs_two_pass": two_pass / el / 1e9,
                                    "hbm_frac_two_pass": two_pass / el / 1e9 / peak,
                                    "coded_requests": int(sum(coded)),
                                    "chunks": st["chunks"], "variant": st["variant"], "grid": st["grid"],
                                    "note": "72 B (PEC) / 84 B (lossy) per cell-update model; the coded two-pass "
                                            "kernels move 76 B (dense 96 / 108 B)"}
        for j in jobs:
            j.close()
        del jobs
        gc.collect()
        torch.cuda.empty_cache()

    # FP64 one at a time, same arrivals, FP32 time step (accuracy reference)
    if not args.serve_no_fp64:
        res64 = {}
        recs64, summ64 = S.serve_one_at_a_time(reqs, np.float64, dt_of=lambda r: S.cfl_dt(r, np.float32),
                                               keep=res64)
        out["plain_fp64_one_at_a_time"] = summ64
        out["speedup_solves_per_hour"] = summ["solves_per_hour"] / summ64["solves_per_hour"]
        out["speedup_tti_p99"] = summ64["tti_p99_s"] / summ["tti_p99_s"]
        wp = [_rel(res32[t]["WP"], res64[t]["WP"]) for t in res32]
        zz = [_rel(res32[t]["Z"], res64[t]["Z"]) for t in res32]
        out["accuracy_vs_fp64"] = {"WP_rel_l2_max": max(wp), "WP_rel_l2_median": float(np.median(wp)),
                                   "Z_rel_l2_max": max(zz), "Z_rel_l2_median": float(np.median(zz)),
                                   "requests_above_1e-4": int(sum(e > 1e-4 for e in wp))}
    if not args.no_cpu:
        rate_all, sample, ncpu = cpu_sample_parallel()
        mean_work = float(np.mean([r.cells * S._steps_estimate(r) for r in reqs]))
        sec = mean_work / (rate_all / ncpu * 1e6)
        out["cpu_baseline"] = {"value": ncpu * 3600.0 / sec, "unit": "solves/h", "cores": ncpu, "kind": "port",
                               "sample": f"{sample}: {rate_all:.2f} M cell-updates/s on {ncpu} cores, extrapolated "
                                         f"to the requests' mean {mean_work:.3e} cell-updates ({sec:.0f} s per solve "
                                         f"and core), {ncpu} single-thread solves at once"}
    print(json.dumps(out), flush=True)


def profile_traffic(name="epass_pillbox_ncu.md"):
    """DRAM bytes per launch (scaled to the full grid) from a committed ncu summary."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    for ln in open(p):
        if ln.startswith("traffic_bytes_per_launch:"):
            try:
                return float(ln.split(":", 1)[1])
            except ValueError:
                return None
    return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--grid", type=int, nargs=3, default=None)
    ap.add_argument("--accuracy", action="store_true", help="FP32 vs FP64 errors on the lossy cavity and the sphere (and the pillbox)")
    ap.add_argument("--accuracy-pillbox", action="store_true")
    ap.add_argument("--serve", action="store_true", help="served wake solves: FP32 pool vs FP64 one at a time")
    ap.add_argument("--serve-count", type=int, default=64)
    ap.add_argument("--serve-budget-gb", type=float, default=4.0)
    ap.add_argument("--serve-load", type=float, default=1.5)
    ap.add_argument("--serve-ref-rate", type=float, default=60.0, help="G cell-updates/s setting the arrival rate")
    ap.add_argument("--serve-chunk", type=int, default=64)
    ap.add_argument("--serve-no-fp64", action="store_true")
    ap.add_argument("--serve-no-saturated", action="store_true")
    ap.add_argument("--serve-fp64-sample", type=int, default=8,
                    help="requests of the sweep run through the plain FP64 path in the default line")
    ap.add_argument("--no-serve", action="store_true", help="default line without the serving block")
    ap.add_argument("--no-dense-roofline", action="store_true", help="default line without the dense fused step timing")
    ap.add_argument("--staging", type=int, default=0, choices=[0, 1, 2],
                    help="with --fused-shape: 0 loads, 1 or 2 TMA plane rings")
    ap.add_argument("--fused-shape", type=int, nargs=4, default=None, metavar=("VEC", "ROWS", "ZSEG", "CTAS"),
                    help="fused step tile shape (skips the autotuner)")
    ap.add_argument("--cpu-workloads", action="store_true",
                    help="CPU oracle rates on the cavity, lossy-cavity and sphere grids (FP64, FP32) and the "
                         "60x60x120 cavity's time-to-impedance")
    ap.add_argument("--cpu-steps", type=int, default=20)
    ap.add_argument("--dense", action="store_true", help="fused step with dense coefficient arrays (no codes)")
    ap.add_argument("--variant", default="auto", choices=["auto", "staged", "direct", "fused"],
                    help="step kernels: auto (the solver default: fused where it applies), direct H/E pass kernels, "
                         "persistent bulk-copy staged pass kernels, or the fused single-pass step")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1 and args.impl == "ours":
        import torch
        torch.distributed.init_process_group("nccl")
    if args.cpu_workloads:
        run_cpu_workloads(args)
    elif args.serve:
        run_serve(args)
    elif args.accuracy or args.accuracy_pillbox:
        run_accuracy(args)
    elif args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world)
    if world > 1 and args.impl == "ours":
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
