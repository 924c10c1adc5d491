"""Time-loop drivers emsolve / wakesolve (wakis/routines.py:17-485).

wakesolve: instead of dumping the 3x3xNz Ez slab to HDF5 every step and integrating it
in Python afterwards, the Ez line integral of the wake potential is accumulated on the
device while the loop runs (FP64, compensated); the tap table (which step feeds which
(s, z) pair) is derived on the host with the post-processor's own expressions, so the
index set is the one WakeSolver.calc_long_WP_3d would use.  The beam current is
evaluated inside the E pass.  Without per-step Python work (no callback, plot or field
monitor) the whole loop runs as CUDA-graph replays with the step number on the device.

emsolve: a PlaneWave / WavePacket source is replayed on the device from per-step
tables; other sources, callbacks and saving run the loop step by step.
"""

import time

import numpy as np
import torch

from . import _native as nat
from .field_monitors import FieldMonitor
from .sources import Beam, PlaneWave, WavePacket


def _step_times(dt, n):
    """t = n*dt for n = 0..n-1 with the scalar types of the reference's `n * self.dt`."""
    if isinstance(dt, np.float32):
        return np.arange(n).astype(np.float32) * dt
    return np.arange(n) * dt


class RoutinesMixin:
    # ------------------------------------------------------------------ emsolve
    def emsolve(self, Nt, source=None, callback=None, save=False, fields=["E"], components=["Abs"], save_every=1,
                subdomain=None, plot=False, plot_every=1, use_etd=False, plot3d=False, **kwargs):
        self.Nt = Nt
        if source is not None:
            self.source = source
        if save:
            self._open_saves(fields, components)
        if plot or plot3d:
            raise NotImplementedError("plotting is not provided")
        abc_axes = self._abc_lo_axes() if self.activate_abc else 0
        self._ctx.call("fit_set_abc", abc_axes)
        # J = sigma*E is taken at the end of the step, before the ABC copy changes plane 0,
        # so on a conductive grid J stays explicit while ABC faces are updated
        self._force_explicit = bool(abc_axes) and self.use_conductivity
        try:
            fast = callback is None and type(source) in (PlaneWave, WavePacket) and not self._force_explicit
            free = source is None and callback is None and not self._force_explicit and self._beam is None
            if fast and Nt > 0:
                self._emsolve_device(Nt, source)
            elif free and Nt > 0:
                self._emsolve_free(Nt)
            else:
                for n in range(Nt):
                    if source is not None:
                        source.update(self, n * self.dt)
                    self.one_step()
                    if callback is not None:
                        callback(self, n * self.dt)
        finally:
            self._ctx.call("fit_set_abc", 0)
            if self._force_explicit:
                # J holds sigma*E of the pre-ABC planes: it stays the truth for the next step
                self._j_state, self._j_zero, self._j_stale = "tensor", False, False
            self._force_explicit = False

    def _emsolve_free(self, Nt):
        """emsolve without a source or callback: the first step through the host path
        (ghost zeroing; explicit J while J is not sigma*E yet), the rest as one device
        loop (CUDA graphs, the fused kernel when selected)."""
        self._advance(self.nstep)
        if Nt == 1:
            return
        if self._choose_mode() != nat.FIT_J_ELIDED:
            for _ in range(Nt - 1):
                self.one_step()
            return
        n0 = self.nstep
        self._device_steps(n0, Nt - 1)
        self.nstep = n0 + Nt - 1
        self._after_device_run()

    def _emsolve_device(self, Nt, source):
        if source.is_first_update:
            source._first(self)
        w = (source.xs.stop if source.xs.stop is not None else self.Nx) - (source.xs.start or 0)
        h = (source.ys.stop if source.ys.stop is not None else self.Ny) - (source.ys.start or 0)
        x0, y0 = source.xs.start or 0, source.ys.start or 0
        if (source.xs.step not in (None, 1)) or (source.ys.step not in (None, 1)) or not isinstance(source.zs, (int, np.integer)):
            # strided or multi-plane sources: step by step through the Field API
            for n in range(Nt):
                source.update(self, n * self.dt)
                self.one_step()
            return
        prof = source.profile(self)
        prof_arr = None
        if prof is not None:
            prof_arr = np.ascontiguousarray(np.broadcast_to(np.asarray(prof, dtype=np.float64), (w, h)).ravel(order="F"))
        tabs = np.array([source.factors(self, n * self.dt) for n in range(Nt)], dtype=np.float64)
        c1, c2, gt = (np.ascontiguousarray(tabs[:, i]) for i in range(3))
        # the first step goes through the Field API as in the reference (source write,
        # then ghost zeroing, then the explicit-J pass if J is not sigma*E yet)
        n0 = self.nstep
        source.update(self, 0 * self.dt)
        self._advance(0)
        if Nt == 1:
            return
        self._ctx.call("fit_set_plane_source", 1, int(source.zs), int(x0), int(x0 + w), int(y0), int(y0 + h),
                       nat.dptr(prof_arr) if prof_arr is not None else None, nat.dptr(c1), nat.dptr(c2),
                       nat.dptr(gt), Nt)
        try:
            if self._choose_mode() != nat.FIT_J_ELIDED:
                raise RuntimeError("J bookkeeping: the device loop needs J = sigma*E or J = 0")
            self._device_steps(1, Nt - 1)
            self.nstep = n0 + Nt
        finally:
            self._ctx.call("fit_set_plane_source", 0, 0, 0, 0, 0, 0, None, None, None, None, 0)
        self._after_device_run()

    # ------------------------------------------------------------------ wakesolve
    def wakesolve(self, wakelength=None, wake=None, callback=None, compute_plane="both", plot=False, plot_func=None,
                  plot_from=None, plot_every=1, plot_until=None, save_J=False, add_space=None,
                  use_field_monitor=False, field_monitor=None, use_edt=None, save_Ez=False, **kwargs):
        """The reference's wakesolve (wakis/routines.py:231-485).  The Ez line history the
        reference always writes to Ez.h5 is recorded on the device only with save_Ez=True
        and written to wake.Ez_file at the end (HDF5 with the reference's datasets when
        h5py is importable, else an .npz archive with the same keys); the wake potential
        itself comes from the device taps either way.  save_J records the J_z slabs on the
        same lines on the device, taken after the beam update and before each step, and
        writes them to Jz.h5 (Jz.npz without h5py) in the working directory, as the
        reference does."""
        if wake is not None:
            self.wake = wake
        if self.wake is None:
            raise AttributeError("Wake solver information not passed to the solver instantiation")
        if wakelength is None:
            wakelength = self.wake.wakelength
        if add_space is not None:
            self.wake.skip_cells = add_space
        if plot:
            raise NotImplementedError("plotting is not provided")
        wake = self.wake
        beam, Nt = self._wake_prepare(wake, wakelength, compute_plane)
        hist = self._start_ez_record(wake, Nt) if save_Ez and Nt > 0 else None
        jhist = self._start_jz_record(wake, Nt) if save_J and Nt > 0 else None
        if self.verbose:
            print("Running electromagnetic time-domain simulation...")
        t0 = time.time()
        monitor = field_monitor if (use_field_monitor and field_monitor is not None) else None
        fast = callback is None and (monitor is None or isinstance(monitor, FieldMonitor))
        if fast and Nt > 0:
            vt = self._wake_device_setup(beam, Nt)
            first = self._wake_first_step(beam)
            if monitor is not None and first > 0:
                monitor.update(self.E, self.dt)
            if monitor is not None and Nt > first:
                self._attach_monitor(monitor, first, Nt - first)
            try:
                self._device_steps(first, Nt - first)
            finally:
                if monitor is not None:
                    self._ctx.call("fit_set_monitor", 0, None, 0, 0, None, 0)
            if monitor is not None:
                monitor.time_index += Nt - first
            self._wake_device_done(vt, Nt)
        else:
            for n in range(Nt):
                beam.update(self, n * self.dt)
                self._advance(n)
                if use_field_monitor and field_monitor is not None:
                    field_monitor.update(self.E, self.dt)
                if callback is not None:
                    callback(self, n * self.dt)
        self.simulationTime = time.time() - t0
        if hist is not None:
            self._ctx.call("fit_set_ez_record", None, 0, None, None, 0, 0)
            self._write_ez(wake, hist, Nt)
        if jhist is not None:
            self._ctx.call("fit_set_jz_record", None, 0, None, None, 0, 0, None)
            self._write_lines("Jz.h5", wake, jhist, Nt)
        wake.solve(compute_plane=compute_plane)
        self.logger.wakeSolver = wake.logger.wakeSolver
        self.logger.wakeSolver["wakelength"] = wakelength
        self.logger.wakeSolver["simulationTime"] = self.simulationTime
        self.logger.solver["Mcell_updates_per_s"] = (self.N * Nt / self.simulationTime / 1e6
                                                     if self.simulationTime > 0 else None)
        self.logger.save_logs()

    # ------------------------------------------------------------------ wakesolve pieces
    def _wake_prepare(self, wake, wakelength, compute_plane):
        """Nt, the Beam and the device tap table of a wake run (wakis/routines.py:340-420)."""
        self.xtest, self.ytest = wake.xtest, wake.ytest
        self.ixt, self.iyt = np.abs(self.x - self.xtest).argmin(), np.abs(self.y - self.ytest).argmin()
        longitudinal = compute_plane.lower() == "longitudinal"
        if longitudinal:
            xx, yy = self.ixt, self.iyt
            lines = [(self.ixt, self.iyt)]
        else:
            xx, yy = slice(self.ixt - 1, self.ixt + 2), slice(self.iyt - 1, self.iyt + 2)
            lines = [(self.ixt + i, self.iyt + j) for i in (-1, 0, 1) for j in (-1, 0, 1)]
        wake.wakelength = wakelength
        self.ti = wake.ti
        self.v = wake.v
        z = self.z
        tmax = (wakelength + self.ti * self.v + (z.max() - z.min())) / self.v
        Nt = int(tmax / self.dt)
        self.tmax, self.Nt = tmax, Nt
        beam = Beam(q=wake.q, sigmaz=wake.sigmaz, beta=wake.beta, xsource=wake.xsource, ysource=wake.ysource)
        # what the reference writes into Ez.h5 besides the field (wakis/routines.py:403-410)
        t = np.arange(0, Nt * self.dt, self.dt)
        wake._attach_run(self, t=t, xf=self.x[xx], yf=self.y[yy], zf=z, dx=self.grid.dx, dy=self.grid.dy,
                         dz=self.grid.dz, lines=lines, nsteps=Nt, longitudinal=longitudinal)
        return beam, Nt

    def _wake_device_setup(self, beam, Nt):
        """Beam and its v*t table on the device for graph-replayed steps 0..Nt-1."""
        beam._first(self)
        self._register_beam(beam)
        vt = np.ascontiguousarray(beam.v * _step_times(self.dt, Nt), dtype=np.float64)
        self._ctx.call("fit_set_beam_vt_table", nat.dptr(vt), Nt)
        self._wake_n0 = self.nstep
        return vt

    def _wake_first_step(self, beam):
        """Takes step 0 from the host when the device loop cannot (first step: ghost
        zeroing; J not equal to what the loss factor assumes).  Returns the next step."""
        if self._choose_mode() != nat.FIT_J_ELIDED or self.step_0:
            beam.update(self, 0 * self.dt)
            self._advance(0)
            return 1
        return 0

    def _wake_device_done(self, vt, Nt):
        self.nstep = self._wake_n0 + Nt
        self._beam_vt = float(vt[-1])
        self._beam_override = not self.use_conductivity
        self._after_device_run()

    # ------------------------------------------------------------------ helpers
    def _start_ez_record(self, wake, Nt):
        """Device buffer (Nt, lines, Nz) of E_z on the wake's integration lines, filled by
        the step prologue before every step."""
        lines = wake._run["lines"]
        hist = torch.empty((Nt, len(lines), self.Nz), dtype=self.E.array.dtype, device=self.E.array.device)
        lx = np.ascontiguousarray([l[0] for l in lines], dtype=np.int32)
        ly = np.ascontiguousarray([l[1] for l in lines], dtype=np.int32)
        self._ctx.call("fit_set_ez_record", nat.C.c_void_p(hist.data_ptr()), len(lines), nat.iptr32(lx),
                       nat.iptr32(ly), 0, int(Nt))
        return hist

    def _start_jz_record(self, wake, Nt):
        """Device buffer (Nt, lines, Nz) of J_z on the wake's lines, filled by the step
        prologue after the beam update and before every step (the reference's save_J dump,
        wakis/routines.py:440-445): the beam current on the beam line, sigma*E elsewhere."""
        lines = wake._run["lines"]
        hist = torch.empty((Nt, len(lines), self.Nz), dtype=self.E.array.dtype, device=self.E.array.device)
        lx = np.ascontiguousarray([l[0] for l in lines], dtype=np.int32)
        ly = np.ascontiguousarray([l[1] for l in lines], dtype=np.int32)
        sz = self.sigma.to_matrix(2)
        sig = np.ascontiguousarray(torch.stack([sz[int(a), int(b), :] for a, b in lines]).double().cpu().numpy())
        self._ctx.call("fit_set_jz_record", nat.C.c_void_p(hist.data_ptr()), len(lines), nat.iptr32(lx),
                       nat.iptr32(ly), 0, int(Nt), nat.dptr(sig))
        return hist

    def _write_lines(self, fname, wake, hist, Nt):
        """A line-history file (Ez.h5, Jz.h5) of the reference from a device-recorded history
        (Nt, lines, Nz); returns the name written."""
        slabs = hist.cpu().numpy()
        shape = (3, 3, self.Nz) if slabs.shape[1] == 9 else (self.Nz,)
        return self._write_history(fname, wake, [slabs[n].reshape(shape) for n in range(Nt)])

    def _write_ez(self, wake, hist, Nt):
        """Ez.h5 of the reference from the device-recorded history (Nt, lines, Nz)."""
        wake.Ez_file = self._write_lines(wake.Ez_file, wake, hist, Nt)

    def _write_history(self, fname, wake, slabs):
        """A line-history file with the reference's datasets (wakis/routines.py:399-427):
        x, y, z, dx, dy, dz, t and one slab per step, '#00000' ...; a slab is
        F[xx, yy, :, 'z'], shape (3, 3, Nz) or (Nz,).  HDF5 when h5py is importable, else
        an .npz archive with the same keys.  Returns the name written."""
        data = {"x": wake.xf, "y": wake.yf, "z": wake.zf, "dx": self.grid.dx, "dy": self.grid.dy,
                "dz": self.grid.dz, "t": wake.t}
        for n, sl in enumerate(slabs):
            data["#" + str(n).zfill(5)] = sl
        try:
            import h5py
        except ImportError:
            h5py = None
        if h5py is not None:
            with h5py.File(fname, "w") as hf:
                for k, v in data.items():
                    hf[k] = v
        else:
            if fname.endswith(".h5"):
                fname = fname[:-3] + ".npz"
            np.savez(fname, **data)
        return fname

    def _attach_monitor(self, monitor, n0, nsteps):
        """FieldMonitor as the epilogue of device-loop steps n0 .. n0+nsteps-1: the phase
        table continues the monitor's own time index."""
        if monitor.dt is None:
            monitor._init(self.E, self.dt)
        ph, single = monitor._pairs(monitor.phases(monitor.time_index, nsteps), self.dtype)
        self._ctx.call("fit_set_monitor", len(monitor.frequencies), nat.dptr(ph), int(n0), int(nsteps),
                       nat.C.c_void_p(monitor._acc.data_ptr()), single)

    def _device_steps(self, n0, nsteps):
        if nsteps <= 0:
            return
        if self.step_0:
            self._set_ghosts_to_0()
            self.step_0 = False
        self._sync_coeffs()
        self._ensure_codes()
        if self._kernels == "fused" and nsteps >= 256:
            self.tune_fused()  # once per grid shape; leaves the fields unchanged
        if self._kernels == "fused":
            self._set_staging()
        self._ctx.call("fit_run", n0, nsteps)
        self._run_steps += nsteps

    def _after_device_run(self):
        self._ctx.call("fit_check_error")  # raises FitError if a kernel gave up a bounded wait
        self._beam_armed = False
        if self.use_conductivity:
            self._j_state = "derived"
            self._j_stale = True
        self._e_zero = False

    def _open_saves(self, fields, components):
        """emsolve(save=True) as the reference runs it (wakis/routines.py:122-146): one HDF5
        file per field and component, 'EAbs.h5', 'Ez.h5', 'Hy.h5', ..., opened for writing;
        then the reference's loop that writes the grid datasets iterates over the file
        NAMES (its dict's keys) and fails on the first one with TypeError, before any
        step.  The same files are created (when h5py is importable) and the same exception
        is raised."""
        try:
            import h5py
        except ImportError:
            h5py = None
        names = []
        for field in fields:
            names += [field + c for c in components] if len(field) == 1 else [field]
        if h5py is not None:
            for nm in names:
                h5py.File(nm + ".h5", "w").close()
        raise TypeError("'str' object does not support item assignment")
