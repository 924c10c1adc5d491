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
        s, it, valid, kskip, nz, nt, w = self._tap_index(nsteps, longitudinal, solver.Nz)
        row_ptr, em, ek0, ecnt = self._tap_csr(it, valid, nsteps)
        lx = np.ascontiguousarray([a for a, _ in lines], dtype=np.int32)
        ly = np.ascontiguousarray([b for _, b in lines], dtype=np.int32)
        dzt = np.ascontiguousarray(w, dtype=np.float64)
        self._run = dict(solver=solver, s=s, nlines=len(lines), lines=list(lines), longitudinal=longitudinal,
                         keep=(lx, ly, row_ptr, em, ek0, ecnt, dzt))
        solver._ctx.call("fit_set_wake_taps", len(lines), nat.iptr32(lx), nat.iptr32(ly), int(kskip), len(s),
                         int(nsteps), nat.iptr64(row_ptr), nat.iptr32(em), nat.iptr32(ek0), nat.iptr32(ecnt),
                         int(nz), nat.dptr(dzt))

    def _wp_index(self, nsaved, counter=False):
        """s and the raw time index it(m, k) exactly as calc_long_WP / calc_long_WP_3d
        evaluate them (wakis/wakeSolver.py:345-369, 449-529), in the reference's loop order:
        k runs over the trimmed z axis, and for a counter-moving test charge (the 3-D
        integral only) loop index k reads z[-k-1] with the time measured from zmax
        (wakis/wakeSolver.py:500-513).  Also the z trim and nt."""
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
        if counter:
            ts = (z[::-1][None, :] - s[:, None]) / (-1 * self.v) - zmax / (-1 * self.v) - self.t[0] + ti
        else:
            ts = (z[None, :] + s[:, None]) / self.v - zmin / self.v - self.t[0] + ti
        it = np.trunc(ts / dt).astype(np.int64)
        return s, it, zz, len(z), nt

    def _loop_dz(self, nz, counter):
        """The dz factor of loop index k: dz[k] of the untrimmed axis (the reference indexes
        dz with the loop index when skip_cells != 0), times -1 for a counter-moving test
        charge."""
        dz = np.asarray(self.dz, dtype=np.float64)[:nz]
        return -1 * dz if counter else dz

    @staticmethod
    def _wrap(it, nt):
        """Ezt[k, it] with Python indexing, as the reference reads it: taps with it >= nt are
        skipped, a negative it counts from the end of the nt recorded steps, and one below
        -nt raises IndexError.  Returns (valid, wrapped index)."""
        valid = it < nt
        itw = np.where(it < 0, it + nt, it)
        if np.any(valid & (itw < 0)):
            bad = int(it[valid & (itw < 0)][0])
            raise IndexError(f"index {bad} is out of bounds for axis 1 with size {nt}")
        return valid, itw

    def _tap_index(self, nsaved, longitudinal, Nz):
        """s, it(m, k) by z index k of the line, the dz factors by z index and the z trim of
        the device taps of a live run.  The sums of a live run are compensated, so only
        the index set and the factors need to be the reference's, not its order."""
        counter = bool(self.counter_moving) and not longitudinal
        s, it, zz, nz, nt = self._wp_index(nsaved, counter)
        if longitudinal and nz != Nz:
            raise ValueError(f"could not broadcast input array from shape ({Nz},) into shape ({nz},): "
                             f"compute_plane='longitudinal' needs skip_cells=0")
        valid, itw = self._wrap(it, nt)
        w = self._loop_dz(nz, counter)
        if counter:  # loop index k reads z index nz-1-k
            valid, itw, w = valid[:, ::-1], itw[:, ::-1], w[::-1]
        kskip = self.skip_cells if self.skip_cells != 0 else 0
        return s, itw, valid, kskip, nz, nt, w

    @staticmethod
    def _tap_csr(it, valid, nsteps):
        """Per-step CSR of (m, k0, cnt): runs of consecutive z indices k that one step feeds
        into one s index m, ordered by step, then m, then k."""
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
        # the runs of one (step, s index) stay adjacent (stable sort): the device sums them
        # in one thread, so a time index that is not monotone in z (wrapped negative
        # indices) needs no special case
        row_ptr = np.searchsorted(gs, np.arange(nsteps + 1), side="left").astype(np.int64)
        return (np.ascontiguousarray(row_ptr), np.ascontiguousarray(gm, dtype=np.int32),
                np.ascontiguousarray(gk, dtype=np.int32), np.ascontiguousarray(cnt, dtype=np.int32))

    def _finalize_device(self, transverse_lines=False):
        """WP_3d (lines x len(s)), WPx and WPy of a live run from the device accumulators.
        With transverse_lines (calc_long_WP_3d), n_transverse_cells other than 1 reads the
        recorded 3x3 lines the way the reference reads its 3x3 Ez slabs,
        Ez[1 + i, 1 + j] for i, j in -n..n with Python indexing: n = 0 keeps the centre
        line alone, and an index past the slab raises the reference's IndexError."""
        r = self._run
        s = r["s"]
        ns = len(s)
        nl = r["nlines"]
        wp3d = np.empty(nl * ns)
        wpx = np.empty(ns)
        wpy = np.empty(ns)
        n = self.n_transverse_cells
        if transverse_lines and nl == 9 and n != 1:
            for i in range(-n, n + 1):
                for j in range(-n, n + 1):
                    for ax, idx in ((0, 1 + i), (1, 1 + j)):
                        if not -3 <= idx < 3:
                            raise IndexError(f"index {idx} is out of bounds for axis {ax} with size 3")
            # n = 0: the centre line only, its own sum divided by q*1e12
            raw = np.empty(nl * ns)
            r["solver"]._ctx.call("fit_read_wake", nat.dptr(raw))
            return s, (raw.reshape(nl, ns)[4] / (self.q * 1e12))[None, :], None, None
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
        Ez[sh0//2 + i, sh1//2 + j, zz] for i, j in -n..n (n = n_transverse_cells, Python
        indexing) for calc_long_WP_3d, whose loop over z runs backwards with negated dz
        for a counter-moving test charge.  The file is closed afterwards, as the reference
        closes it."""
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
        counter = bool(self.counter_moving) and not longitudinal
        s, it, zz, nz, nt = self._wp_index(len(keys), counter)
        nc = self.n_transverse_cells
        ofs = [(1, 1)] if longitudinal else [(i, j) for i in range(-nc, nc + 1) for j in range(-nc, nc + 1)]
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
        valid, itw = self._wrap(it, nt)
        table = np.ascontiguousarray(np.where(valid, itw, -1).T, dtype=np.int32)  # (nz, ns), loop order
        dz = self._loop_dz(nz, counter)
        eloop = ezt[:, ::-1, :] if counter else ezt  # loop index k reads z index nz-1-k
        if not longitudinal and nc >= 1:
            dxf, dyf = np.diff(self.xf), np.diff(self.yf)
            wp3d, wpx, wpy = nat.wake_history(eloop, table, dz, self.q * 1e12, s[2] - s[1],
                                              dxf[nc - 1] + dxf[nc], dyf[nc - 1] + dyf[nc])
        else:
            wp3d, wpx, wpy = nat.wake_history(eloop, table, dz, self.q * 1e12)
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
            s, wp3d, wpx, wpy = self._finalize_device(transverse_lines=True)
        else:
            s, wp3d, wpx, wpy, _ = self._history_wp(False)
        n = self.n_transverse_cells
        self.s = s
        self.WP_3d = wp3d.reshape(2 * n + 1, 2 * n + 1, len(s))
        self.WP = self.WP_3d[n, n, :]
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
        if self.n_transverse_cells < 1:  # the reference reads WP_3d[i0 + 1, ...] of a 1x1 WP_3d
            raise IndexError("index 1 is out of bounds for axis 0 with size 1")
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
        """Spectrum of a wake function, returned as [f, Z] with the conventions of the
        reference's utility (wakis/wakeSolver.py:1185-1253).  The time axis is wake[0] when
        wake is a list [t, W], else s/c, else t (AttributeError when none is given).  With
        fmax the record is first resampled by linear interpolation onto a uniform axis of
        step 1/(2 fmax) over [t.min(), t.max()); without it fmax = 1/dt.  The transform has
        2*samples points (zero padding) or one point per sample, and the frequencies
        0 <= f < fmax are kept, scaled by 2/len(record)."""
        if isinstance(wake, list):
            t, wake = wake[0], wake[1]
        if s is not None:
            t = s / c_light
        elif t is None:
            raise AttributeError('Provide time data through parameter "t" [s] or "s" [m]')
        record, step = WakeSolver._uniform_record(np.asarray(t), np.asarray(wake),
                                                  None if fmax is None else 1 / fmax / 2)
        if fmax is None:
            fmax = 1 / step
        npts = record.shape[0]
        nfft = npts if samples is None else 2 * samples
        spectrum = np.fft.fft(record, n=nfft)
        freqs = np.fft.fftfreq(nfft, step)
        band = (freqs >= 0) & (freqs < fmax)
        if verbose:
            print(f"    * Number of samples = {int(band.sum())}")
        return [freqs[band], spectrum[band] / npts * 2]

    @staticmethod
    def calc_wake_from_impedance(impedance, f=None, tmax=None, samples=None, pad=0, verbose=True):
        """Wake function of an impedance, returned as [t, W] with the conventions of the
        reference's utility (wakis/wakeSolver.py:1255-1315): impedance is [f, Z] when it
        has two entries, else Z with the frequencies in f (AttributeError without them).
        With tmax, Z is resampled onto a uniform frequency axis of step 1/tmax; without it
        tmax = 1/df.  W(t_i) = -Re(sum_b Z_b exp(-2 pi i b (i+1) / n)) over n = samples
        points (len(Z) when samples is None), that is the transform advanced by one sample,
        on t = n points evenly spaced over [0, tmax]."""
        if len(impedance) == 2:
            f, Z = impedance[0], impedance[1]
        elif f is None:
            raise AttributeError('Provide frequency data through parameter "f"')
        else:
            Z = impedance
        Z, step = WakeSolver._uniform_record(np.asarray(f), np.asarray(Z), None if tmax is None else 1 / tmax)
        if tmax is None:
            tmax = 1 / step
        n = Z.shape[0] if samples is None else samples
        spectrum = np.fft.fft(Z, n=n)
        wake = -spectrum.real[(np.arange(n) + 1) % n]
        return [np.linspace(0, tmax, n), wake]

    @staticmethod
    def _uniform_record(axis, values, spacing):
        """(values, mean step) of a sampled record; with a spacing the record is first
        interpolated linearly onto np.arange(axis.min(), axis.max(), spacing)."""
        if spacing is None:
            return values, np.mean(axis[1:] - axis[:-1])
        uni = np.arange(axis.min(), axis.max(), spacing)
        return np.interp(uni, axis, values), np.mean(uni[1:] - uni[:-1])

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

    # the text files a run with save=True writes, in the order load_results reads them,
    # with the attributes their two columns go to (None: the column is not kept)
    _RESULT_FILES = (("lambda.txt", None, "lambdas"), ("WPx.txt", None, "WPx"), ("WPy.txt", None, "WPy"),
                     ("WP.txt", "s", "WP"), ("spectrum.txt", None, "lambdaf"), ("Zx.txt", None, "Zx"),
                     ("Zy.txt", None, "Zy"), ("Z.txt", "f", "Z"))

    def load_results(self, folder=None):
        """Reads back the results a run with save=True wrote (wakis/wakeSolver.py:1477-1511):
        each file's two columns through read_txt; f is stored as its absolute value, the
        wakelength is the last s, and folder and Ez_file (folder + 'Ez.h5') are set."""
        if folder is None:
            if self.folder is None:
                raise Exception("[!] Please provide a folder path")
            folder = self.folder
        base = folder if folder.endswith("/") else folder + "/"
        for fname, xattr, yattr in self._RESULT_FILES:
            xcol, ycol = self.read_txt(base + fname).values()
            if xattr is not None:
                setattr(self, xattr, xcol)
            setattr(self, yattr, ycol)
        self.f = np.abs(self.f)
        self.wakelength = self.s[-1]
        self.folder = base
        self.Ez_file = base + "Ez.h5"

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
