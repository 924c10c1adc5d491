"""WakeSolver: wake potential and impedance from the Ez line integral
(wakis/wakeSolver.py:19-874, 1185-1315, 1526-1538, 1713-1727).

Same constructor, attributes and results (s, WP, WP_3d, WPx, WPy, f, Z, Zx, Zy,
lambdas, lambdaf).  The difference is where the integral is evaluated: when a
wakis_gb300 solver ran ``wakesolve``, the integral
    WP[m] = sum_k Ez(x_line, y_line, z_k, t = it(m, k)) * dz[k] / (q*1e12)
was accumulated on the device during the time loop from a tap table built here with
the reference's own index expression
    it(m, k) = int(((z_k + s_m)/v - zmin/v - t_0 + ti) / (t_2 - t_1)),  used when it < nt,
so the result is the reference's, including its quirks: the 3x3 lines share one
accumulator that is divided by q*1e12 after each line, dz is indexed on the untrimmed
axis when skip_cells != 0, and the post-processing injection time uses
ti = 8.5489*sigmaz/(sqrt(beta)*v).  The transverse wake and both impedances are then
computed on the device in FP64 (prefix sums, central differences, direct DFT).
"""

import os
import time

import numpy as np
from scipy.constants import c as c_light

from . import _native as nat
from .logger import Logger


class WakeSolver:
    def __init__(self, wakelength=None, q=1e-9, sigmaz=1e-3, beta=1.0, xsource=0.0, ysource=0.0, xtest=0.0,
                 ytest=0.0, chargedist=None, ti=None, fmax=None, compute_plane="both", skip_cells=0,
                 add_space=None, Ez_file=None, save=True, results_folder="results/", verbose=1,
                 counter_moving=False):
        self.verbose = verbose
        self.log("Initializing Wakefield parameters...")
        t0 = time.time()
        self.q = q
        self.sigmaz = sigmaz
        self.beta = beta
        self.v = self.beta * c_light
        self.xsource, self.ysource = xsource, ysource
        self.xtest, self.ytest = xtest, ytest
        self.chargedist = chargedist
        self.ti = ti
        self.fmax = self.v / (3.0 * self.sigmaz) if fmax is None else fmax
        self.skip_cells = skip_cells
        self.compute_plane = compute_plane
        self.DE_model = None
        self.counter_moving = counter_moving
        if counter_moving:
            raise NotImplementedError("counter_moving test charges are not provided")
        if add_space is not None:
            self.skip_cells = add_space
        if ti is not None:
            self.ti = ti
        else:
            self.ti = 8.548921333333334 * self.sigmaz / (np.sqrt(self.beta) * self.v)
        self.Ez_file = Ez_file
        self.Ez_hf = None
        self.Ezt = None
        self.t = None
        self.xf, self.yf, self.zf = None, None, None
        self.x, self.y, self.z = None, None, None
        self.wakelength = wakelength
        self.s = None
        self.lambdas = None
        self.WP = None
        self.WP_3d = None
        self.n_transverse_cells = 1
        self.WPx, self.WPy = None, None
        self.f = None
        self.Z = None
        self.Zx, self.Zy = None, None
        self.lambdaf = None
        self.logger = Logger()
        self.save = save
        self.folder = results_folder
        if not self.folder.endswith("/"):
            self.folder += "/"
        if self.Ez_file is None:
            self.Ez_file = self.folder + "Ez.h5"
        if self.save:
            os.makedirs(self.folder, exist_ok=True)
        self._run = None
        self.assign_logs()
        self.log(f"Total solver initialization time: {time.time() - t0} s")

    # ------------------------------------------------------------------ device run
    def _attach_run(self, solver, t, xf, yf, zf, dx, dy, dz, lines, nsteps, longitudinal):
        """Called by wakesolve before the time loop: records what the reference stores in
        Ez.h5 and installs the tap table on the solver's device context."""
        self.t = np.asarray(t)
        self.xf, self.yf, self.zf = np.atleast_1d(np.asarray(xf)), np.atleast_1d(np.asarray(yf)), np.asarray(zf)
        self.dx, self.dy, self.dz = np.asarray(dx), np.asarray(dy), np.asarray(dz)
        s, it, valid, kskip, nz, nt = self._tap_index(nsteps, longitudinal, solver.Nz)
        row_ptr, em, ek0, ecnt = self._tap_csr(it, valid, nsteps)
        lx = np.ascontiguousarray([a for a, _ in lines], dtype=np.int32)
        ly = np.ascontiguousarray([b for _, b in lines], dtype=np.int32)
        dzt = np.ascontiguousarray(self.dz[:nz], dtype=np.float64)
        self._run = dict(solver=solver, s=s, nlines=len(lines), lines=list(lines), longitudinal=longitudinal,
                         keep=(lx, ly, row_ptr, em, ek0, ecnt, dzt))
        solver._ctx.call("fit_set_wake_taps", len(lines), nat.iptr32(lx), nat.iptr32(ly), int(kskip), len(s),
                         int(nsteps), nat.iptr64(row_ptr), nat.iptr32(em), nat.iptr32(ek0), nat.iptr32(ecnt),
                         int(nz), nat.dptr(dzt))

    def _wp_index(self, nsaved):
        """s and the raw time index it(m, k) exactly as calc_long_WP_3d / calc_long_WP
        evaluate them (wakis/wakeSolver.py:345-369, 449-529), the z trim and nt."""
        nt = len(self.t)
        dt = self.t[2] - self.t[1]
        ti = self.ti
        zmax = np.max(self.zf)
        zmin = np.min(self.zf)
        zz = slice(self.skip_cells, -self.skip_cells) if self.skip_cells != 0 else np.s_[:]
        z = self.zf[zz]
        if self.wakelength is not None:
            wakelength = self.wakelength
        else:
            wakelength = nt * dt * self.v - (zmax - zmin) - ti * self.v
            self.wakelength = wakelength
        s = np.arange(-self.ti * self.v, wakelength, dt * self.v)
        nt = min(nt, nsaved)
        ts = (z[None, :] + s[:, None]) / self.v - zmin / self.v - self.t[0] + ti
        it = np.trunc(ts / dt).astype(np.int64)
        return s, it, zz, len(z), nt

    def _tap_index(self, nsaved, longitudinal, Nz):
        """s and it(m, k) of the device taps of a live run."""
        s, it, zz, nz, nt = self._wp_index(nsaved)
        if longitudinal and nz != Nz:
            raise ValueError(f"could not broadcast input array from shape ({Nz},) into shape ({nz},): "
                             f"compute_plane='longitudinal' needs skip_cells=0")
        valid = it < nt
        if np.any(valid & (it < 0)):
            raise NotImplementedError("negative time index in the wake integral (a tap before t=0)")
        kskip = self.skip_cells if self.skip_cells != 0 else 0
        return s, it, valid, kskip, nz, nt

    @staticmethod
    def _tap_csr(it, valid, nsteps):
        """Per-step CSR of (m, k0, cnt): for a fixed s-index m, it(m, k) is non-decreasing in
        k, so the k that one step feeds form one contiguous run, and adding the runs in step
        order adds the terms in the reference's k order."""
        M, K = np.nonzero(valid)
        st = it[M, K]
        if M.size == 0:
            return (np.zeros(nsteps + 1, dtype=np.int64), np.zeros(0, np.int32), np.zeros(0, np.int32),
                    np.zeros(0, np.int32))
        brk = np.ones(M.size, dtype=bool)
        brk[1:] = (M[1:] != M[:-1]) | (st[1:] != st[:-1]) | (K[1:] != K[:-1] + 1)
        starts = np.nonzero(brk)[0]
        cnt = np.diff(np.append(starts, M.size))
        gm, gk, gs = M[starts], K[starts], st[starts]
        order = np.lexsort((gm, gs))
        gm, gk, gs, cnt = gm[order], gk[order], gs[order], cnt[order]
        dup = (gs[1:] == gs[:-1]) & (gm[1:] == gm[:-1])
        if np.any(dup):
            raise NotImplementedError("wake tap index not monotone in z")
        row_ptr = np.searchsorted(gs, np.arange(nsteps + 1), side="left").astype(np.int64)
        return (np.ascontiguousarray(row_ptr), np.ascontiguousarray(gm, dtype=np.int32),
                np.ascontiguousarray(gk, dtype=np.int32), np.ascontiguousarray(cnt, dtype=np.int32))

    def _finalize_device(self):
        r = self._run
        s = r["s"]
        ns = len(s)
        nl = r["nlines"]
        wp3d = np.empty(nl * ns)
        wpx = np.empty(ns)
        wpy = np.empty(ns)
        if nl == 9:
            ds = s[2] - s[1]
            dxf, dyf = np.diff(self.xf), np.diff(self.yf)
            dxs, dys = dxf[0] + dxf[1], dyf[0] + dyf[1]
        else:
            ds, dxs, dys = 1.0, 1.0, 1.0
        r["solver"]._ctx.call("fit_wake_finalize", nat.C.c_double(self.q * 1e12), nat.C.c_double(ds),
                              nat.C.c_double(dxs), nat.C.c_double(dys), nat.dptr(wp3d), nat.dptr(wpx),
                              nat.dptr(wpy))
        return s, wp3d.reshape(nl, ns), wpx, wpy

    # ------------------------------------------------------------------ solve
    def solve(self, compute_plane=None, **kwargs):
        if compute_plane is None:
            compute_plane = self.compute_plane
        for key, val in kwargs.items():
            setattr(self, key, val)
        t0 = time.time()
        if compute_plane.lower() in ["both", "transverse"]:
            self.calc_long_WP_3d()
            self.calc_trans_WP()
            self.calc_long_Z()
            self.calc_trans_Z()
        elif compute_plane.lower() == "longitudinal":
            self.calc_long_WP()
            self.calc_long_Z()
        self.log("Calculation terminated in %ds" % (time.time() - t0))

    def _history_wp(self, longitudinal, Ezt=None):
        """The wake integral of an Ez file: without a live run, calc_long_WP and
        calc_long_WP_3d read the per-step slabs of ``Ez_file`` (HDF5, or the .npz archive
        with the same keys) and evaluate the integral on the device in the reference's
        operation order, so s and WP / WP_3d equal the reference's bit for bit
        (wakis/wakeSolver.py:333-413, 446-540).  Slab lines follow the reference: the 1-D
        slab itself, or Ez[sh0//2 + 1, sh1//2 + 1, zz] for calc_long_WP on 3-D slabs,
        Ez[sh0//2 + i, sh1//2 + j, zz] for the 3x3 lines of calc_long_WP_3d.  The file is
        closed afterwards, as the reference closes it."""
        if Ezt is not None:
            self.Ezt = Ezt
            if self.Ez_hf is None:
                # the reference keeps Ezt and then assembles it again from the unopened file
                raise AttributeError("'NoneType' object has no attribute 'keys'")
        elif self.Ez_hf is None:
            self.read_Ez()
        hf = self.Ez_hf
        keys = sorted(k for k in hf.keys() if isinstance(k, str) and k.startswith("#"))
        if not keys:
            raise IndexError("list index out of range")
        s, it, zz, nz, nt = self._wp_index(len(keys))
        ofs = [(1, 1)] if longitudinal else [(i, j) for i in (-1, 0, 1) for j in (-1, 0, 1)]
        ezt = np.zeros((len(ofs), nz, nt))
        ndim = np.ndim(hf[keys[0]])
        for n in range(nt):
            E = np.asarray(hf[keys[n]])
            if longitudinal and ndim == 1:
                ezt[0, :, n] = E
            elif longitudinal and ndim != 3:
                continue  # the reference leaves Ezt at zero for other slab shapes
            else:
                for li, (i, j) in enumerate(ofs):
                    ezt[li, :, n] = E[E.shape[0] // 2 + i, E.shape[1] // 2 + j, zz]
        valid = it < nt
        itw = np.where(it < 0, it + nt, it)
        if np.any(valid & (itw < 0)):
            bad = int(it[valid & (itw < 0)][0])
            raise IndexError(f"index {bad} is out of bounds for axis 1 with size {nt}")
        table = np.ascontiguousarray(np.where(valid, itw, -1).T, dtype=np.int32)  # (nz, ns)
        dz = np.asarray(self.dz, dtype=np.float64)[:nz]
        if len(ofs) == 9:
            dxf, dyf = np.diff(self.xf), np.diff(self.yf)
            wp3d, wpx, wpy = nat.wake_history(ezt, table, dz, self.q * 1e12, s[2] - s[1], dxf[0] + dxf[1],
                                              dyf[0] + dyf[1])
        else:
            wp3d, wpx, wpy = nat.wake_history(ezt, table, dz, self.q * 1e12)
        hf.close()
        self.Ez_hf = None
        return s, wp3d, wpx, wpy, ezt

    def calc_long_WP(self, Ezt=None, **kwargs):
        for key, val in kwargs.items():
            setattr(self, key, val)
        if self._run is not None:
            s, wp3d, _, _ = self._finalize_device()
        else:
            s, wp3d, _, _, ezt = self._history_wp(True, Ezt)
            self.Ezt = ezt[0]
        self.s = s
        self.WP = wp3d[0]
        if self.save:
            self._savetxt("WP.txt", self.s, self.WP, "WP [V/pC]", "   s [m]")

    def calc_long_WP_3d(self, **kwargs):
        for key, val in kwargs.items():
            setattr(self, key, val)
        if self._run is not None:
            s, wp3d, wpx, wpy = self._finalize_device()
        else:
            s, wp3d, wpx, wpy, _ = self._history_wp(False)
        self.s = s
        self.WP_3d = wp3d.reshape(3, 3, len(s))
        self.WP = self.WP_3d[1, 1, :]
        self._wpxy = (wpx, wpy)
        if self.save:
            self._savetxt("WP.txt", self.s, self.WP, "WP [V/pC]", "   s [m]")

    def calc_trans_WP(self, **kwargs):
        """Panofsky-Wenzel transverse wake (wakis/wakeSolver.py:553-626), computed on the
        device together with the line combination."""
        for key, val in kwargs.items():
            setattr(self, key, val)
        if getattr(self, "_wpxy", None) is None:
            self.calc_long_WP_3d()
        self.WPx, self.WPy = self._wpxy
        if self.save:
            self._savetxt("WPx.txt", self.s, self.WPx, "WP [V/pC]", "   s [m]")
            self._savetxt("WPy.txt", self.s, self.WPy, "WP [V/pC]", "   s [m]")

    def _dft_setup(self, samples, fmax):
        ds = np.mean(self.s[1:] - self.s[:-1])
        fmax = self.fmax if fmax is None else fmax
        N = int((self.v / ds) // fmax * samples)
        ffft = np.fft.fftfreq(N, ds / self.v)
        mask = np.logical_and(ffft >= 0, ffft < fmax)
        bins = np.nonzero(mask)[0]
        if bins.size and not np.array_equal(bins, np.arange(bins.size)):
            raise RuntimeError("non-contiguous frequency bins")
        return ds, N, ffft, mask, bins.size

    def _dft(self, signals, N, nb):
        x = np.atleast_2d(np.asarray(signals, dtype=np.float64))
        x = x[:, :N]  # np.fft.fft(a, n) crops inputs longer than n
        return nat.dft(x, N, 0, nb)

    def calc_long_Z(self, samples=1001, fmax=None, **kwargs):
        """Longitudinal impedance (wakis/wakeSolver.py:628-720): the n-point zero-padded
        DFT is evaluated directly, in FP64 on the device, at the kept bins 0 <= f < fmax."""
        for key, val in kwargs.items():
            setattr(self, key, val)
        if self.lambdas is None and self.chargedist is not None:
            self.calc_lambdas()
        elif self.lambdas is None and self.chargedist is None:
            self.calc_lambdas_analytic()
        ds, N, ffft, mask, nb = self._dft_setup(samples, fmax)
        X = self._dft([self.lambdas * self.v, self.WP * 1e12], N, nb)
        lambdaf = X[0] * ds
        WPf = X[1] * ds
        self.f = ffft[mask]
        self.Z = -WPf / lambdaf
        self.lambdaf = lambdaf
        if self.save:
            self._savetxt("Z.txt", self.f, self.Z, "Z [Ohm]", "   f [Hz]")
            self._savetxt("spectrum.txt", self.f, self.lambdaf, "Charge distribution spectrum [C/s]", "   f [Hz]")

    def calc_trans_Z(self, samples=1001, fmax=None):
        """Transverse impedances (wakis/wakeSolver.py:722-785)."""
        ds, N, ffft, mask, nb = self._dft_setup(samples, fmax)
        X = self._dft([self.lambdas * self.v, self.WPx * 1e12, self.WPy * 1e12], N, nb)
        lambdaf = X[0] * ds
        self.Zx = 1j * (X[1] * ds) / lambdaf
        self.Zy = 1j * (X[2] * ds) / lambdaf
        self.fx = ffft[mask]
        self.fy = ffft[mask]
        if self.save:
            self._savetxt("Zx.txt", self.fx, self.Zx, "Zx [Ohm]", "   f [Hz]")
            self._savetxt("Zy.txt", self.fy, self.Zy, "Zy [Ohm]", "   f [Hz]")

    def calc_lambdas(self, **kwargs):
        """Charge distribution lambda(s) from data (wakis/wakeSolver.py:787-840)."""
        for key, val in kwargs.items():
            setattr(self, key, val)
        if type(self.chargedist) is str:
            d = self.read_txt(self.chargedist)
            keys = list(d.keys())
            z, chargedist = d[keys[0]], d[keys[1]]
        elif type(self.chargedist) is dict:
            keys = list(self.chargedist.keys())
            z, chargedist = self.chargedist[keys[0]], self.chargedist[keys[1]]
        else:
            chargedist = self.chargedist
            if self.z is not None and len(self.z) == len(chargedist):
                z = self.z
            elif self.zf is not None and len(self.zf) == len(chargedist):
                z = self.zf
            else:
                raise ValueError("Dimension error: check input dimensions")
        self.lambdas = np.interp(self.s, z, chargedist / self.q)
        if self.save:
            self._savetxt("lambda.txt", self.s, self.lambdas, "Charge distribution [C/m]", "   s [Hz]")

    def calc_lambdas_analytic(self, **kwargs):
        """Gaussian lambda(s) (wakis/wakeSolver.py:842-874)."""
        for key, val in kwargs.items():
            setattr(self, key, val)
        self.lambdas = 1 / (self.sigmaz * np.sqrt(2 * np.pi)) * np.exp(-(self.s ** 2) / (2 * self.sigmaz ** 2))
        if self.save:  # the reference labels this file's s column "[Hz]"
            self._savetxt("lambda.txt", self.s, self.lambdas, "Charge distribution [C/m]", "   s [Hz]")

    # ------------------------------------------------------------------ utilities
    @staticmethod
    def calc_impedance_from_wake(wake, s=None, t=None, fmax=None, samples=None, verbose=True):
        """FFT of a wake function (wakis/wakeSolver.py:1185-1253)."""
        if type(wake) is list:
            t = wake[0]
            wake = wake[1]
        if s is not None:
            t = s / c_light
        elif s is None and t is None:
            raise AttributeError('Provide time data through parameter "t" [s] or "s" [m]')
        dt = np.mean(t[1:] - t[:-1])
        if fmax is not None:
            aux = np.arange(t.min(), t.max(), 1 / fmax / 2)
            wake = np.interp(aux, t, wake)
            dt = np.mean(aux[1:] - aux[:-1])
        else:
            fmax = 1 / dt
        Wfft = np.fft.fft(wake, n=2 * samples) if samples is not None else np.fft.fft(wake)
        ffft = np.fft.fftfreq(len(Wfft), dt)
        mask = np.logical_and(ffft >= 0, ffft < fmax)
        return [ffft[mask], Wfft[mask] / len(wake) * 2]

    @staticmethod
    def calc_wake_from_impedance(impedance, f=None, tmax=None, samples=None, pad=0, verbose=True):
        """Inverse transform of an impedance (wakis/wakeSolver.py:1255-1315)."""
        if len(impedance) == 2:
            f, Z = impedance[0], impedance[1]
        elif f is None:
            raise AttributeError('Provide frequency data through parameter "f"')
        else:
            Z = impedance
        df = np.mean(f[1:] - f[:-1])
        if tmax is not None:
            aux = np.arange(f.min(), f.max(), 1 / tmax)
            Z = np.interp(aux, f, Z)
        else:
            tmax = 1 / df
        wake = np.real(-1 * np.fft.fft(Z, n=samples))
        wake = np.roll(wake, -1)
        return [np.linspace(0, tmax, len(wake)), wake]

    def read_Ez(self, filename=None, return_value=False):
        """Opens an Ez line history (wakis/wakeSolver.py:1317-1364): an HDF5 file as the
        reference writes it, or the .npz archive with the same keys that
        SolverFIT3D.wakesolve(save_Ez=True) writes without h5py.  Sets xf, yf, zf, dx, dy,
        dz and t; the per-step slabs '#00000', ... stay in Ez_hf."""
        if filename is None:
            filename = self.Ez_file
        if str(filename).endswith(".npz"):
            hf = np.load(filename)
        else:
            try:
                import h5py
            except ImportError:
                raise ImportError("reading an HDF5 Ez file needs h5py; wakesolve(save_Ez=True) writes an .npz "
                                  "archive with the same keys when h5py is missing") from None
            hf = h5py.File(filename, "r")
        self.log(f"Reading Ez file {filename}")
        self.Ez_hf = hf
        self.Ez_file = filename
        keys = set(hf.keys())
        for key, attr in (("x", "xf"), ("y", "yf"), ("z", "zf"), ("dx", "dx"), ("dy", "dy"), ("dz", "dz"),
                          ("t", "t")):
            if key in keys:
                setattr(self, attr, np.array(hf[key]))
        if return_value:
            return hf

    def read_txt(self, txt, skiprows=2, delimiter=None, usecols=None):
        """Columns of a text result file as a dict (wakis/wakeSolver.py:1366-1420): keys are
        the header's column names with their units ("s[m]", "WP[V/pC]"), or 0, 1, ...
        when the file has no such header; complex columns are read as complex128."""
        try:
            load = np.loadtxt(txt, skiprows=skiprows, delimiter=delimiter, usecols=usecols)
        except Exception:
            self.log(f"[!] Using dtype=np.complex128 to read {txt}", level=2)
            load = np.loadtxt(txt, skiprows=skiprows, delimiter=delimiter, usecols=usecols, dtype=np.complex128)
        try:
            with open(txt) as f:
                header = f.readline()
            header = header.replace(" ", "").replace("#", "").replace("\n", "").split("]")
            d = {}
            for i in range(len(load[0, :])):
                d[header[i] + "]"] = load[:, i]
        except Exception:
            self.log("[!] Using integer keys since no header was found", level=2)
            d = {}
            for i in range(len(load[0, :])):
                d[i] = load[:, i]
        return d

    def save_txt(self, f_name, x_data=None, y_data=None, x_name="X [-]", y_name="Y [-]"):
        """Two-column text file f_name(.txt) with the reference's header
        (wakis/wakeSolver.py:1422-1475)."""
        if f_name.endswith(".txt"):
            f_name = f_name[:-4]
        if x_data is not None and y_data is not None:
            np.savetxt(f_name + ".txt", np.c_[x_data, y_data], header="   " + x_name + " " * 20 + y_name + "\n" + "-" * 48)
        else:
            self.log("[!] txt not saved, please provide x_data and y_data")

    def load_results(self, folder=None):
        """Reads the results a run with save=True wrote (wakis/wakeSolver.py:1477-1511):
        lambdas, WPx, WPy, s, WP, lambdaf, Zx, Zy, f (absolute value) and Z; sets
        wakelength = s[-1], folder and Ez_file = folder + 'Ez.h5'."""
        if folder is None and self.folder is None:
            raise Exception("[!] Please provide a folder path")
        elif folder is None:
            folder = self.folder
        if not folder.endswith("/"):
            folder = folder + "/"
        _, self.lambdas = self.read_txt(folder + "lambda.txt").values()
        _, self.WPx = self.read_txt(folder + "WPx.txt").values()
        _, self.WPy = self.read_txt(folder + "WPy.txt").values()
        self.s, self.WP = self.read_txt(folder + "WP.txt").values()
        _, self.lambdaf = self.read_txt(folder + "spectrum.txt").values()
        _, self.Zx = self.read_txt(folder + "Zx.txt").values()
        _, self.Zy = self.read_txt(folder + "Zy.txt").values()
        self.f, self.Z = self.read_txt(folder + "Z.txt").values()
        self.f = np.abs(self.f)
        self.wakelength = self.s[-1]
        self.folder = folder
        self.Ez_file = folder + "Ez.h5"

    def _savetxt(self, name, a, b, label, xlabel):
        np.savetxt(self.folder + name, np.c_[a, b], header=xlabel + " " * 20 + label + "\n" + "-" * 48)

    def copy(self):
        obj = type(self).__new__(self.__class__)
        obj.__dict__.update(self.__dict__)
        return obj

    def log(self, txt, level=1):
        if level <= self.verbose:
            print(txt) if level == 1 else print("\x1b[2;37m" + txt + "\x1b[0m")

    def assign_logs(self):
        for k in ("ti", "q", "sigmaz", "beta", "xsource", "ysource", "xtest", "ytest", "chargedist", "skip_cells"):
            self.logger.wakeSolver[k] = getattr(self, k)
        self.logger.wakeSolver["results_folder"] = self.folder
