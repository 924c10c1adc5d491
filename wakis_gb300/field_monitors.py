"""FieldMonitor: running DFT of the electric field (wakis/field_monitors.py:14-116).

Same interface as the reference: ``FieldMonitor(frequencies)``, ``update(E, dt)``,
``get_components()`` and the attributes ``frequencies``, ``time_index``, ``dt``,
``shape``, ``xp`` and ``Ex_acc / Ey_acc / Ez_acc`` (complex128, shape
``(n_freq, Nx, Ny, Nz)``).  The accumulators live on the field's device (``xp`` is
torch, as the reference's are cupy arrays on its GPU path) in one buffer laid out
[component][frequency][flat cell], which the library's monitor kernel updates.  The
phases exp(-2j*pi*f*t), t = time_index*dt, are evaluated on the host with the
reference's expression and types (complex64 when t is float32, as for an FP32 solver's
dt), and the update uses the reference's operation order and product precision, so the
accumulators equal the reference's bit for bit for the same fields.

``SolverFIT3D.wakesolve(use_field_monitor=True, field_monitor=monitor)`` keeps the
device loop: the monitor runs as an epilogue kernel after every step.
"""

import ctypes as C

import numpy as np

from . import _native as nat


class FieldMonitor:
    def __init__(self, frequencies):
        self.frequencies = np.array(frequencies)
        self.time_index = 0
        self.dt = None
        self.shape = None
        self.xp = None
        self._acc = None

    # ------------------------------------------------------------------ accumulators
    def _view(self, c):
        if self._acc is None:
            return None
        nx, ny, nz = self.shape
        return self._acc[c].reshape(len(self.frequencies), nz, ny, nx).permute(0, 3, 2, 1)

    @property
    def Ex_acc(self):
        return self._view(0)

    @property
    def Ey_acc(self):
        return self._view(1)

    @property
    def Ez_acc(self):
        return self._view(2)

    def get_components(self):
        return {"Ex": self.Ex_acc, "Ey": self.Ey_acc, "Ez": self.Ez_acc}

    def _init(self, E, dt):
        import torch
        self.dt = dt
        self.shape = (E.Nx, E.Ny, E.Nz)
        self.xp = E.xp
        n = E.Nx * E.Ny * E.Nz
        self._acc = torch.zeros((3, len(self.frequencies), n), dtype=torch.complex128, device=E.array.device)

    def phases(self, first, count):
        """(count, n_freq) complex phases of updates first .. first+count-1, evaluated as
        the reference does: t = time_index * dt in the type that product has (float32
        for an FP32 solver's dt), then exp(-2j*pi*f*t) -- complex64 for a float32 t,
        as numpy gives."""
        tdt = np.asarray(int(first) * self.dt).dtype
        t = np.arange(first, first + count).astype(tdt) * tdt.type(self.dt)
        cols = [np.exp(-2j * np.pi * f * t) for f in self.frequencies]
        return np.stack(cols, axis=1) if cols else np.empty((count, 0), dtype=np.complex128)

    @staticmethod
    def _pairs(ph, field_dtype):
        """(re, im) float64 pairs of the phases and the library's single flag: products
        rounded to FP32 when numpy would multiply an FP32 field by complex64 phases."""
        single = int(ph.dtype == np.complex64 and np.dtype(field_dtype) == np.float32)
        return np.ascontiguousarray(ph.astype(np.complex128)).view(np.float64).reshape(-1), single

    # ------------------------------------------------------------------ update
    def update(self, E, dt):
        """Adds E * exp(-2j*pi*f*t) to the accumulators, t = time_index*dt (dt fixed at
        the first call), and advances time_index."""
        import torch
        if self.dt is None:
            self._init(E, dt)
        f64 = E.array.dtype == torch.float64
        ph, single = self._pairs(self.phases(self.time_index, 1), np.float64 if f64 else np.float32)
        stream = torch.cuda.current_stream(E.array.device).cuda_stream
        rc = nat.load().fit_monitor_update(C.c_void_p(E.array.data_ptr()), nat.FIT_F64 if f64 else nat.FIT_F32,
                                           int(self._acc.shape[2]), len(self.frequencies), nat.dptr(ph),
                                           C.c_void_p(self._acc.data_ptr()), single, C.c_void_p(stream))
        nat.check(rc)
        self.time_index += 1
