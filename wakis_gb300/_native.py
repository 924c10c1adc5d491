"""ctypes binding of libwakis_fit.so (the C ABI declared in include/wakis_fit.h).

There is no CPU fallback: importing the solver without the library, or calling it
without a CUDA device, raises.  The library is built in-tree by wakis_gb300.build.
"""

import ctypes as C
import os
import threading

import numpy as np

from . import build as _build

FIT_F32, FIT_F64 = 0, 1
FIT_BC = {"periodic": 0, "pec": 1, "electric": 1, "pml": 2, "pmc": 3, "magnetic": 3, "abc": 4}
FIT_J_ELIDED, FIT_J_EXPLICIT = 0, 1

FIT_ERR_TIMEOUT = -4
FIT_ERR_BUDGET = -7
FIT_ERR_CANCELLED = -8
_ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "invalid state", -4: "timeout", -5: "out of memory",
           -6: "no device", -7: "over the pool budget", -8: "cancelled"}


class FitError(RuntimeError):
    """A libwakis_fit call returned a negative status."""

    def __init__(self, code, msg):
        super().__init__(f"libwakis_fit error {code} ({_ERRORS.get(code, '?')}): {msg}")
        self.code = code


class FitGridDesc(C.Structure):
    _fields_ = [("nx", C.c_int64), ("ny", C.c_int64), ("nz", C.c_int64), ("dtype", C.c_int32),
                ("use_conductivity", C.c_int32), ("bc_lo", C.c_int32 * 3), ("bc_hi", C.c_int32 * 3),
                ("device", C.c_int32), ("reserved", C.c_int32), ("E", C.c_void_p), ("H", C.c_void_p),
                ("J", C.c_void_p)]


class FitPoolDone(C.Structure):
    _fields_ = [("tag", C.c_int64), ("steps", C.c_int64), ("status", C.c_int32), ("reserved", C.c_int32),
                ("t_submit_ms", C.c_double), ("t_start_ms", C.c_double), ("t_done_ms", C.c_double)]


class FitPoolStats(C.Structure):
    _fields_ = [("chunks", C.c_int64), ("cell_updates", C.c_int64), ("budget_bytes", C.c_int64),
                ("reserved_bytes", C.c_int64), ("active", C.c_int32), ("queued", C.c_int32),
                ("max_active", C.c_int32), ("chunk_steps", C.c_int32), ("variant", C.c_int32 * 3),
                ("grid", C.c_int32 * 3), ("busy_ms", C.c_double), ("fused_cell_updates", C.c_int64),
                ("fused_variant", C.c_int32 * 3), ("fused_grid", C.c_int32 * 3)]


_P = C.c_void_p
_D = C.POINTER(C.c_double)
_I32 = C.POINTER(C.c_int32)
_I64 = C.POINTER(C.c_int64)

_SIGS = {
    "fit_ctx_create": (C.POINTER(FitGridDesc), C.POINTER(C.c_void_p)),
    "fit_ctx_destroy": (_P,),
    "fit_last_error": (_P, C.c_char_p, C.c_int64),
    "fit_set_stream": (_P, _P),
    "fit_set_fields": (_P, _P, _P, _P),
    "fit_set_metrics": (_P, _D, _D, _D, _D, _D, _D),
    "fit_set_coeffs": (_P, C.c_double, _P, _P, _P),
    "fit_enable_explicit_j": (_P,),
    "fit_zero_ghosts": (_P,),
    "fit_set_beam": (_P, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_double, C.c_double,
                     C.c_double, C.c_double, _D, _D),
    "fit_set_beam_vt": (_P, C.c_double),
    "fit_set_beam_vt_table": (_P, _D, C.c_int64),
    "fit_set_plane_source": (_P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, _D, _D, _D,
                             _D, C.c_int64),
    "fit_set_abc": (_P, C.c_int32),
    "fit_set_wake_taps": (_P, C.c_int32, _I32, _I32, C.c_int32, C.c_int32, C.c_int64, _I64, _I32, _I32, _I32,
                          C.c_int32, _D),
    "fit_reset_wake": (_P,),
    "fit_read_wake": (_P, _D),
    "fit_step": (_P, C.c_int64, C.c_int32),
    "fit_run": (_P, C.c_int64, C.c_int64),
    "fit_materialize_J": (_P, _P, C.c_int32),
    "fit_wake_finalize": (_P, C.c_double, C.c_double, C.c_double, C.c_double, _D, _D, _D),
    "fit_dft": (_D, C.c_int32, C.c_int64, C.c_int64, C.c_int64, C.c_int32, _D),
    "fit_wake_history": (_D, C.c_int32, C.c_int64, C.c_int32, _I32, C.c_int32, _D, C.c_double, C.c_double,
                         C.c_double, C.c_double, _D, _D, _D),
    "fit_time_kernels": (_P, C.c_int32, _D),
    "fit_check_error": (_P,),
    "fit_dft_noalloc": (_P, C.c_int32, C.c_int64, C.c_int64, C.c_int64, C.c_int32, _P, _P),
    "fit_set_kernel_variant": (_P, C.c_int32),
    "fit_time_fused": (_P, C.c_int32, _D),
    "fit_set_fused_shape": (_P, C.c_int32, C.c_int32, C.c_int32, C.c_int32),
    "fit_set_fused_staging": (_P, C.c_int32, C.c_int32),
    "fit_set_wait_limit": (_P, C.c_int64),
    "fit_set_coeff_codes": (_P, C.c_int32, C.POINTER(C.c_int32)),
    "fit_monitor_update": (_P, C.c_int32, C.c_int64, C.c_int32, _D, _P, C.c_int32, _P),
    "fit_set_monitor": (_P, C.c_int32, _D, C.c_int64, C.c_int64, _P, C.c_int32),
    "fit_set_ez_record": (_P, _P, C.c_int32, _I32, _I32, C.c_int64, C.c_int64),
    "fit_set_jz_record": (_P, _P, C.c_int32, _I32, _I32, C.c_int64, C.c_int64, _D),
    "fit_pool_create": (C.c_int32, C.c_int64, C.c_int32, C.c_int32, C.POINTER(C.c_void_p)),
    "fit_pool_destroy": (_P,),
    "fit_pool_last_error": (_P, C.c_char_p, C.c_int64),
    "fit_pool_reserve": (_P, C.c_int64),
    "fit_pool_release": (_P, C.c_int64),
    "fit_pool_submit": (_P, _P, C.c_int64, C.c_int64, C.c_int64),
    "fit_pool_poll": (_P, C.POINTER(FitPoolDone), C.c_int32, C.c_int32),
    "fit_pool_cancel": (_P, C.c_int64),
    "fit_pool_stats": (_P, C.POINTER(FitPoolStats)),
    "fit_pool_tune": (_P, C.c_int32, C.c_int32),
    "fit_pool_tune_fused": (_P, C.c_int32, C.c_int32),
    "fit_version": (C.c_char_p, C.c_int64),
    "fit_launch_count": (),
}

_lib = None
_lock = threading.Lock()


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Loads (building first if needed) and returns the ctypes library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if build_if_missing and (not os.path.exists(path) or _build.needs_build()):
            _build.build()
        if not os.path.exists(path):
            raise ImportError(f"libwakis_fit.so not found at {path}; run `python -m wakis_gb300.build`")
        lib = C.CDLL(path)
        for name, args in _SIGS.items():
            f = getattr(lib, name)
            f.argtypes = list(args)
            f.restype = C.c_int64 if name == "fit_launch_count" else C.c_int
        _lib = lib
        return lib


def exported_symbols():
    return list(_SIGS)


def last_error(ctx=None):
    buf = C.create_string_buffer(1024)
    load().fit_last_error(ctx, buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc, ctx=None):
    if rc != 0:
        raise FitError(rc, last_error(ctx))


def dptr(a):
    """ctypes double* of a C-contiguous float64 numpy array (kept alive by the caller)."""
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_D)


def iptr32(a):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_I32)


def iptr64(a):
    assert a.dtype == np.int64 and a.flags.c_contiguous
    return a.ctypes.data_as(_I64)


def launch_count():
    return int(load().fit_launch_count())


def dft(signals, n, b0, nb):
    """FP64 DFT of real signals (nsig, len) at bins b0..b0+nb-1 of an n-point transform."""
    x = np.ascontiguousarray(np.atleast_2d(np.asarray(signals, dtype=np.float64)))
    out = np.empty((x.shape[0], nb, 2), dtype=np.float64)
    rc = load().fit_dft(dptr(x), x.shape[0], x.shape[1], int(n), int(b0), int(nb), dptr(out))
    check(rc)
    return out[..., 0] + 1j * out[..., 1]


def wake_history(ezt, it, dz, qscale, ds=1.0, dxf=1.0, dyf=1.0):
    """Wake integral of a recorded Ez line history on the device: ezt (nlines, nz, nt)
    FP64, it (nz, ns) int32 (-1 = no tap), dz (nz,).  Returns (wp3d (nlines, ns), wpx,
    wpy); wpx and wpy are None unless the lines form a square of odd side >= 3."""
    ezt = np.ascontiguousarray(ezt, dtype=np.float64)
    it = np.ascontiguousarray(it, dtype=np.int32)
    dz = np.ascontiguousarray(dz, dtype=np.float64)
    nl, nz, nt = ezt.shape
    ns = it.shape[1]
    if it.shape[0] != nz or dz.shape != (nz,):
        raise ValueError("wake_history: shapes of ezt, it and dz do not agree")
    wp3d = np.empty((nl, ns))
    wpx, wpy = np.empty(ns), np.empty(ns)
    rc = load().fit_wake_history(dptr(ezt), nl, nt, nz, iptr32(it), ns, dptr(dz), float(qscale), float(ds),
                                 float(dxf), float(dyf), dptr(wp3d), dptr(wpx), dptr(wpy))
    check(rc)
    side = int(round(nl ** 0.5))
    square = side >= 3 and side % 2 == 1 and side * side == nl
    return (wp3d, wpx, wpy) if square else (wp3d, None, None)


class Context:
    """Owns one FitCtx.  All device pointers passed in are torch tensors kept alive here."""

    def __init__(self, nx, ny, nz, dtype, use_conductivity, bc_low, bc_high, E, H, J, device=0):
        self.lib = load()
        d = FitGridDesc()
        d.nx, d.ny, d.nz = nx, ny, nz
        d.dtype = FIT_F64 if dtype == np.float64 else FIT_F32
        d.use_conductivity = int(bool(use_conductivity))
        for a in range(3):
            d.bc_lo[a] = bc_code(bc_low[a])
            d.bc_hi[a] = bc_code(bc_high[a])
        d.device = device
        d.E, d.H, d.J = E.data_ptr(), H.data_ptr(), J.data_ptr()
        self._keep = [E, H, J]
        h = C.c_void_p()
        check(self.lib.fit_ctx_create(C.byref(d), C.byref(h)))
        self.h = h

    def call(self, name, *args):
        rc = getattr(self.lib, name)(self.h, *args)
        if rc != 0:
            raise FitError(rc, last_error(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.lib.fit_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Pool:
    """Owns one FitPool (the serving executor of FP32 wake solves on one device)."""

    def __init__(self, budget_bytes, chunk_steps=64, ctas_per_sm=0, device=0):
        self.lib = load()
        h = C.c_void_p()
        rc = self.lib.fit_pool_create(int(device), int(budget_bytes), int(chunk_steps), int(ctas_per_sm),
                                      C.byref(h))
        if rc != 0:
            raise FitError(rc, self._err(None))
        self.h = h

    def _err(self, h):
        buf = C.create_string_buffer(1024)
        self.lib.fit_pool_last_error(h, buf, len(buf))
        return buf.value.decode(errors="replace")

    def _check(self, rc):
        if rc < 0:
            raise FitError(rc, self._err(self.h))
        return rc

    def reserve(self, nbytes):
        """True when nbytes fit in the budget now (and are reserved), False otherwise."""
        rc = self.lib.fit_pool_reserve(self.h, int(nbytes))
        if rc == FIT_ERR_BUDGET:
            return False
        self._check(rc)
        return True

    def release(self, nbytes):
        self._check(self.lib.fit_pool_release(self.h, int(nbytes)))

    def submit(self, ctx, n0, nsteps, tag):
        rc = self.lib.fit_pool_submit(self.h, ctx.h, int(n0), int(nsteps), int(tag))
        if rc != 0:
            raise FitError(rc, last_error(ctx.h))

    def poll(self, wait_ms=0, max_n=64):
        out = (FitPoolDone * max_n)()
        n = self._check(self.lib.fit_pool_poll(self.h, out, max_n, int(wait_ms)))
        return [dict(tag=d.tag, steps=d.steps, status=d.status, t_submit_ms=d.t_submit_ms,
                     t_start_ms=d.t_start_ms, t_done_ms=d.t_done_ms) for d in out[:n]]

    def cancel(self, tag):
        """Cancels a queued or running solve: poll() reports it with status
        FIT_ERR_CANCELLED once no chunk in flight steps it (or FIT_OK if its last steps
        were already in flight)."""
        self._check(self.lib.fit_pool_cancel(self.h, int(tag)))

    def stats(self):
        s = FitPoolStats()
        self._check(self.lib.fit_pool_stats(self.h, C.byref(s)))
        out = {name: getattr(s, name) for name, _ in FitPoolStats._fields_}
        out["variant"] = {4: s.variant[0], 2: s.variant[1], 1: s.variant[2]}
        out["grid"] = {4: s.grid[0], 2: s.grid[1], 1: s.grid[2]}
        out["fused_variant"] = {4: s.fused_variant[0], 2: s.fused_variant[1], 1: s.fused_variant[2]}
        out["fused_grid"] = {4: s.fused_grid[0], 2: s.fused_grid[1], 1: s.fused_grid[2]}
        return out

    def tune(self, vec, ctas_per_sm):
        """Selects the compiled pass-kernel variant of one vector-width class."""
        self._check(self.lib.fit_pool_tune(self.h, int(vec), int(ctas_per_sm)))

    def tune_fused(self, vec, ctas_per_sm):
        """Selects the compiled variant of the pooled fused step of one vector-width class."""
        self._check(self.lib.fit_pool_tune_fused(self.h, int(vec), int(ctas_per_sm)))

    def close(self):
        if getattr(self, "h", None):
            self.lib.fit_pool_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def bc_code(name):
    key = str(name).lower()
    if key not in FIT_BC:
        raise ValueError(f"boundary condition {name!r} is not supported (periodic, pec/electric, pml, "
                         f"pmc/magnetic, abc)")
    return FIT_BC[key]
