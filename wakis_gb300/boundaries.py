"""Boundary handling of SolverFIT3D (wakis/boundaries.py:14-404).

The curl-matrix edits of the reference become face codes of the native context: PEC and
PML faces zero tangential E columns, PMC faces zero tangential H rows, periodic and
high ABC faces copy the first dual length / inverse dual area onto the last one
(applied by libwakis_fit from the codes).  Here: flag handling, the graded-conductivity
PML slabs, and the ABC plane snapshots of emsolve.
"""

import numpy as np
import torch
from scipy.constants import epsilon_0

_KNOWN = ("periodic", "pec", "electric", "pml", "pmc", "magnetic", "abc")


class BCsMixin:
    def _check_bcs(self):
        lo = [b.lower() for b in self.bc_low]
        hi = [b.lower() for b in self.bc_high]
        for b in lo + hi:
            if b not in _KNOWN:
                raise ValueError(f"boundary condition {b!r} is not supported: {_KNOWN}")
        if "abc" in lo or "abc" in hi:
            self.activate_abc = True
        if "pml" in lo or "pml" in hi:
            self.activate_pml = True
            self.use_conductivity = True

    def _initialize_PML(self):
        """Graded-conductivity PML slabs (wakis/boundaries.py:190-305): in each slab
        ieps = 1/eps_0 and sigma = geomspace(1.0 -> 5e-3) S/m with the outermost cell at
        1.0; slabs are written x-lo, y-lo, z-lo, x-hi, y-hi, z-hi (later ones win)."""
        self.pml_lo = 5.0e-3
        self.pml_hi = 1.0
        self.pml_func = np.geomspace
        self.pml_eps_r = 1.0
        n = self.n_pml
        prof_lo = self.pml_func(self.pml_hi, self.pml_lo, n)
        prof_hi = self.pml_func(self.pml_lo, self.pml_hi, n)
        lo = [b.lower() for b in self.bc_low]
        hi = [b.lower() for b in self.bc_high]
        ieps_pml = 1 / epsilon_0

        def write(axis, idx, sig):
            for d in range(3):
                for f, val in ((self.ieps, ieps_pml), (self.sigma, sig)):
                    m = f.to_matrix(d)
                    sl = [slice(None)] * 3
                    sl[axis] = idx
                    m[tuple(sl)] = val

        for a in range(3):
            if lo[a] == "pml":
                for i in range(n):
                    write(a, i, 0.0 + 1 * float(prof_lo[i]))
        for a in range(3):
            if hi[a] == "pml":
                for i in range(1, n + 1):
                    write(a, -i, 0.0 + 1 * float(prof_hi[-i]))

    def _abc_lo_axes(self):
        lo = [b.lower() for b in self.bc_low]
        hi = [b.lower() for b in self.bc_high]
        for a in range(3):
            if lo[a] == "abc" and hi[a] == "abc":
                # the reference's snapshot dict of that axis loses its low entries
                raise KeyError("xyz"[a] + "lo")
        n = (self.Nx, self.Ny, self.Nz)
        for a in range(3):
            if lo[a] == "abc" and n[a] < 2:
                # the reference's update copies plane 1 of that axis (wakis/boundaries.py:363-404)
                raise IndexError(f"index 1 is out of bounds for axis {a} with size {n[a]}")
        return sum(1 << a for a in range(3) if lo[a] == "abc")

    def get_abc(self):
        """Boundary-plane snapshots (copies) for update_abc (wakis/boundaries.py:307-361)."""
        E_abc, H_abc = {}, {}
        lo = [b.lower() for b in self.bc_low]
        hi = [b.lower() for b in self.bc_high]
        planes = {0: (np.s_[1, :, :], np.s_[-1, :, :]), 1: (np.s_[:, 1, :], np.s_[:, -1, :]),
                  2: (np.s_[:, :, 1], np.s_[:, :, -1])}
        for a in range(3):
            for side, name in ((0, "lo"), (1, "hi")):
                if (lo if side == 0 else hi)[a] == "abc":
                    E_abc[a], H_abc[a] = {}, {}
                    for d in "xyz":
                        sl = planes[a][side]
                        E_abc[a][d + name] = self.E[sl + (d,)]
                        H_abc[a][d + name] = self.H[sl + (d,)]
        return E_abc, H_abc

    def update_abc(self, E_abc, H_abc):
        """Writes the snapshots onto the exterior planes (wakis/boundaries.py:363-404)."""
        lo = [b.lower() for b in self.bc_low]
        hi = [b.lower() for b in self.bc_high]
        planes = {0: (np.s_[0, :, :], np.s_[-1, :, :]), 1: (np.s_[:, 0, :], np.s_[:, -1, :]),
                  2: (np.s_[:, :, 0], np.s_[:, :, -1])}
        for side, name, flags in ((0, "lo", lo), (1, "hi", hi)):
            for a in range(3):
                if flags[a] == "abc":
                    for d in "xyz":
                        sl = planes[a][side]
                        self.E[sl + (d,)] = E_abc[a][d + name]
                        self.H[sl + (d,)] = H_abc[a][d + name]
