"""GridFIT3D: rectilinear primal/dual grid and solid masks.

Mirrors the reference's constructor (wakis/gridFIT3D.py:31-261) and metric definitions
(wakis/gridFIT3D.py:263-305):
  * primal edge lengths L (dx[i], dy[j], dz[k]) and inverse areas iA = 1/(L_p L_q);
  * dual edge lengths tL from cell midpoints with the last midpoint duplicated, so
    tL[-1] = 0, and inverse dual areas itA = 1/(tL_p tL_q), 0 where the area is 0.
The metrics are separable, so they are held as 1-D arrays; ``L``, ``iA``, ``tL`` and
``itA`` are also available as full Fields (built on demand, host memory).

Solids: ``stl_solids`` maps a name to an analytic solid, either a callable
``f(X, Y, Z) -> bool array`` or a boolean mask over the (Nx, Ny, Nz) cells (C order, the
order in which the solver reshapes ``grid.grid[key]``).  Callables are evaluated at the
cell corners with the reference's default 'legacy' rule (a cell is inside when any of
its 8 corners is inside) or, with ``stl_method='center'``, at the cell centres.  STL
files need a mesh voxeliser (VTK), which this package does not ship: passing a file
name raises.  ``stl_materials`` takes library keys or [eps_r, mu_r(, sigma)] lists.
"""

import time

import numpy as np

from .field import Field
from .logger import Logger
from .materials import material_colors, material_lib


class _MaskStore(dict):
    """Per-solid cell masks, ``grid.grid[key]`` -> flat bool array (C order)."""


class GridFIT3D:
    def __init__(self, xmin=None, xmax=None, ymin=None, ymax=None, zmin=None, zmax=None, Nx=None, Ny=None,
                 Nz=None, x=None, y=None, z=None, use_mpi=False, use_mesh_refinement=False,
                 refinement_method="insert", refinement_tol=1e-8, snap_points=None, snap_tol=1e-5,
                 snap_solids=None, stl_solids=None, stl_materials=None, stl_rotate=[0.0, 0.0, 0.0],
                 stl_translate=[0.0, 0.0, 0.0], stl_scale=1.0, stl_colors=None, stl_tol=1e-3,
                 stl_method="legacy", load_from_h5=None, verbose=1):
        t0 = time.time()
        self.logger = Logger()
        self.verbose = verbose
        self.use_mpi = use_mpi
        if use_mpi:
            raise NotImplementedError("use_mpi: z-slab MPI decomposition is not provided; run one domain "
                                      "per GPU")
        if load_from_h5 is not None:
            self.load_from_h5(load_from_h5)
            return
        if x is not None and y is not None and z is not None:
            self.x, self.y, self.z = (np.asarray(x, dtype=float), np.asarray(y, dtype=float),
                                      np.asarray(z, dtype=float))
            self.Nx, self.Ny, self.Nz = len(self.x) - 1, len(self.y) - 1, len(self.z) - 1
            self.xmin, self.xmax = self.x[0], self.x[-1]
            self.ymin, self.ymax = self.y[0], self.y[-1]
            self.zmin, self.zmax = self.z[0], self.z[-1]
        elif all(v is not None for v in [xmin, xmax, ymin, ymax, zmin, zmax]):
            self.xmin, self.xmax = xmin, xmax
            self.ymin, self.ymax = ymin, ymax
            self.zmin, self.zmax = zmin, zmax
            self.Nx, self.Ny, self.Nz = int(Nx), int(Ny), int(Nz)
            self.x = np.linspace(self.xmin, self.xmax, self.Nx + 1)
            self.y = np.linspace(self.ymin, self.ymax, self.Ny + 1)
            self.z = np.linspace(self.zmin, self.zmax, self.Nz + 1)
        else:
            raise ValueError("[!] Error initializing GridFIT3D:\n"
                             "  - Provide grid axis arrays: x, y, z\n"
                             "  - OR domain extents and number of cells: xmin, xmax, ymin, ymax, zmin, zmax, "
                             "Nx, Ny, Nz\n  - OR load from a file using load_from_h5")
        self.use_mesh_refinement = use_mesh_refinement
        self.refinement_method = refinement_method
        self.snap_points = snap_points
        self.snap_tol = snap_tol
        self.snap_solids = snap_solids
        if use_mesh_refinement:
            self._refine_from_snaps(snap_points, stl_solids, refinement_method, refinement_tol)
        self.dx, self.dy, self.dz = np.diff(self.x), np.diff(self.y), np.diff(self.z)
        self.update_logger(["Nx", "Ny", "Nz", "dx", "dy", "dz"])
        self.update_logger(["xmin", "xmax", "ymin", "ymax", "zmin", "zmax"])
        self.stl_solids = stl_solids
        self.stl_materials = stl_materials
        self.stl_rotate, self.stl_translate, self.stl_scale = stl_rotate, stl_translate, stl_scale
        self.stl_colors = stl_colors
        self.stl_tol = stl_tol
        self.stl_method = stl_method
        self.update_logger(["stl_solids", "stl_materials"])
        self._compute_grid()
        if stl_solids is not None:
            self._prepare_stl_dicts()
            self._mark_cells_in_stl(stl_method)
        self.gridInitializationTime = time.time() - t0
        self.update_logger(["gridInitializationTime"])

    # ------------------------------------------------------------------ metrics
    # ------------------------------------------------------------------ mesh refinement
    def _refine_from_snaps(self, snap_points, stl_solids, method, tol):
        """use_mesh_refinement (wakis/gridFIT3D.py:204-217, 654-699, 861-920): each axis is
        re-spaced by refine_axis so that it passes through the snap coordinates.  The
        reference derives those from the STL solids' feature edges (points lying in the
        x = 0, y = 0 and z = 0 planes, rounded to 5 decimals, plus the domain bounds),
        which needs VTK: that extraction is not provided.  Given snap_points (an (n, 3)
        array standing for those edge points), the same derivation runs on them; the
        reference itself raises AttributeError there, as it reads x_snaps, which only the
        STL extraction sets."""
        if snap_points is None:
            if stl_solids is not None:
                raise NotImplementedError("use_mesh_refinement extracts snap points from STL feature edges, which "
                                          "needs VTK; pass snap_points, or refined x, y, z arrays")
            raise AttributeError("'GridFIT3D' object has no attribute 'x_snaps'")
        pts = np.atleast_2d(np.asarray(snap_points, dtype=float))
        for a, name in enumerate("xyz"):
            lo, hi = getattr(self, name + "min"), getattr(self, name + "max")
            snaps = np.unique(np.concatenate(([lo], np.unique(np.round(pts[:, a], 5)), [hi])))
            setattr(self, name + "_snaps", snaps)
        self.x = self.refine_axis(self.xmin, self.xmax, self.Nx + 1, self.x_snaps, method=method, tol=tol)
        self.y = self.refine_axis(self.ymin, self.ymax, self.Ny + 1, self.y_snaps, method=method, tol=tol)
        self.z = self.refine_axis(self.zmin, self.zmax, self.Nz + 1, self.z_snaps, method=method, tol=tol)
        self.Nx, self.Ny, self.Nz = len(self.x) - 1, len(self.y) - 1, len(self.z) - 1

    @staticmethod
    def _spread_residuals(u, anchor, pinned):
        """The three residuals refine_axis minimises over the normalised node positions u
        (wakis/gridFIT3D.py:795-808): pinned nodes that moved (weight 1000, squared), gaps
        below the uniform gap 1/(n-1) (squared shortfall), and 10 x the standard deviation
        of the gaps."""
        gaps = np.diff(u)
        moved = np.sum((u[pinned] - anchor[pinned]) ** 2) * 1000
        small = gaps[gaps < 1 / (len(u) - 1)]
        short = np.sum((1 / (len(u) - 1) - small) ** 2)
        return np.hstack([moved, short, np.std(gaps) * 10])

    def refine_axis(self, xmin, xmax, Nx, x_snaps, method="insert", tol=1e-12):
        """Nodes of an axis on [xmin, xmax] that pass through the snap coordinates x_snaps with
        gaps as even as possible (wakis/gridFIT3D.py:771-859).  Positions are normalised
        to [0, 1] and a start is built: 'insert' merges the snaps into Nx - len(x_snaps)
        uniform nodes; 'neighbor' moves, for each snap, the first of Nx uniform nodes
        within half a gap onto it.  Then scipy's least_squares (dogbox within [0, 1],
        arctan loss, 3-point Jacobian, tolerances tol) minimises _spread_residuals, which
        keeps the snap nodes in place.  'subdivision' raises the reference's
        UnboundLocalError (its start is never assigned); other names raise ValueError."""
        from scipy.optimize import least_squares
        snaps = (x_snaps - xmin) / (xmax - xmin)
        if method == "insert":
            start = np.unique(np.append(snaps, np.linspace(0, 1, Nx - len(snaps))))
        elif method == "neighbor":
            start = np.linspace(0, 1, Nx)
            half = np.diff(start)[0] / 2
            for v in snaps:
                near = np.isclose(start, v, rtol=0.0, atol=half)
                if near.any():
                    start[np.argmax(near)] = v
        elif method == "subdivision":
            raise UnboundLocalError("cannot access local variable 'x' where it is not associated with a value")
        else:
            raise ValueError(f"Method {method} not supported. Use 'insert', 'neighbor' or 'subdivision'.")
        pinned = np.isin(start, snaps)
        fit = least_squares(self._spread_residuals, x0=start.copy(), bounds=(0, 1), jac="3-point", method="dogbox",
                            loss="arctan", gtol=tol, ftol=tol, xtol=tol, verbose=0, args=(start.copy(), pinned.copy()))
        return fit.x * (xmax - xmin) + xmin

    def _compute_grid(self):
        self.grid = _MaskStore()
        tx = np.append((self.x[1:] + self.x[:-1]) / 2, 0.0)
        tx[-1] = tx[-2]
        ty = np.append((self.y[1:] + self.y[:-1]) / 2, 0.0)
        ty[-1] = ty[-2]
        tz = np.append((self.z[1:] + self.z[:-1]) / 2, 0.0)
        tz[-1] = tz[-2]
        self.tx, self.ty, self.tz = tx, ty, tz
        # dual edge lengths: last entry 0 (duplicated midpoint)
        self.tdx, self.tdy, self.tdz = np.diff(tx), np.diff(ty), np.diff(tz)
        self._fields = {}

    def _field_from(self, fx, fy, fz):
        f = Field(self.Nx, self.Ny, self.Nz)
        for d, m in enumerate((fx, fy, fz)):
            f.from_matrix(m, d)
        return f

    def _metric(self, name):
        if name in self._fields:
            return self._fields[name]
        X = np.broadcast_to(self.dx[:, None, None], (self.Nx, self.Ny, self.Nz))
        Y = np.broadcast_to(self.dy[None, :, None], (self.Nx, self.Ny, self.Nz))
        Z = np.broadcast_to(self.dz[None, None, :], (self.Nx, self.Ny, self.Nz))
        tX = np.broadcast_to(self.tdx[:, None, None], X.shape)
        tY = np.broadcast_to(self.tdy[None, :, None], X.shape)
        tZ = np.broadcast_to(self.tdz[None, None, :], X.shape)

        def safe_inv(a):
            return np.divide(1.0, a, out=np.zeros_like(a), where=a != 0)

        if name == "L":
            f = self._field_from(X, Y, Z)
        elif name == "iA":
            f = self._field_from(np.divide(1.0, Y * Z), np.divide(1.0, X * Z), np.divide(1.0, X * Y))
        elif name == "tL":
            f = self._field_from(tX, tY, tZ)
        else:
            f = self._field_from(safe_inv(tY * tZ), safe_inv(tX * tZ), safe_inv(tX * tY))
        self._fields[name] = f
        return f

    L = property(lambda self: self._metric("L"))
    iA = property(lambda self: self._metric("iA"))
    tL = property(lambda self: self._metric("tL"))
    itA = property(lambda self: self._metric("itA"))

    # ------------------------------------------------------------------ solids
    def _prepare_stl_dicts(self):
        if not isinstance(self.stl_solids, dict):
            self.stl_solids = {"Solid 1": self.stl_solids}
        if not isinstance(self.stl_materials, dict):
            if isinstance(self.stl_materials, (str, list, tuple)):
                self.stl_materials = {k: self.stl_materials for k in self.stl_solids}
            else:
                raise Exception("[!] Attribute `stl_materials` must contain a string or a dictionary")
        if not isinstance(self.stl_colors, dict):
            self.stl_colors = {k: (self.stl_colors if isinstance(self.stl_colors, str) else "other")
                               for k in self.stl_solids}
        for key in self.stl_solids:
            mat = self.stl_materials[key]
            if isinstance(mat, str):
                m = material_lib[mat.lower()]
                self.stl_materials[key] = list(m)
                self.stl_colors[key] = material_colors.get(mat.lower(), self.stl_colors.get(key))

    def _mark_cells_in_stl(self, method="legacy"):
        for key, solid in self.stl_solids.items():
            self.grid[key] = self.solid_mask(solid, method).reshape(-1)

    def solid_mask(self, solid, method=None):
        """Boolean (Nx, Ny, Nz) cell mask of one solid."""
        method = (method or self.stl_method).lower()
        shape = (self.Nx, self.Ny, self.Nz)
        if isinstance(solid, str):
            raise NotImplementedError(f"STL file {solid!r}: voxelising a mesh needs VTK; pass an analytic "
                                      f"solid f(X, Y, Z) -> bool or a boolean (Nx, Ny, Nz) mask")
        if callable(solid):
            if method == "center":
                xc = self.x[:-1] + self.dx / 2
                yc = self.y[:-1] + self.dy / 2
                zc = self.z[:-1] + self.dz / 2
                X, Y, Z = np.meshgrid(xc, yc, zc, indexing="ij")
                return np.asarray(solid(X, Y, Z), dtype=bool)
            X, Y, Z = np.meshgrid(self.x, self.y, self.z, indexing="ij")
            inside = np.asarray(solid(X, Y, Z), dtype=bool)
            m = np.zeros(shape, dtype=bool)
            for a in (0, 1):
                for b in (0, 1):
                    for c in (0, 1):
                        m |= inside[a:a + self.Nx, b:b + self.Ny, c:c + self.Nz]
            return m
        if type(solid).__module__.startswith("torch"):
            # a torch bool tensor (e.g. built on the GPU for large grids) stays where it is
            if solid.numel() != self.Nx * self.Ny * self.Nz:
                raise ValueError(f"solid mask has {solid.numel()} cells, the grid has "
                                 f"{self.Nx * self.Ny * self.Nz}")
            return solid.reshape(shape).bool()
        m = np.asarray(solid, dtype=bool)
        if m.size != self.Nx * self.Ny * self.Nz:
            raise ValueError(f"solid mask has {m.size} cells, the grid has {self.Nx * self.Ny * self.Nz}")
        return m.reshape(shape)

    # ------------------------------------------------------------------ persistence
    def save_to_h5(self, filename="grid.h5"):
        """Saves axes, solids and masks.  Writes HDF5 when h5py is importable, otherwise an
        .npz archive at the same path."""
        data = {"x": self.x, "y": self.y, "z": self.z}
        for k in self.grid:
            data["mask:" + k] = np.asarray(self.grid[k])
            mat = (self.stl_materials or {}).get(k)
            if mat is not None:
                data["material:" + k] = np.asarray(mat, dtype=float)
        try:
            import h5py
        except ImportError:
            with open(filename, "wb") as fh:
                np.savez(fh, **data)
            return
        with h5py.File(filename, "w") as hf:
            for k, v in data.items():
                hf[k] = v

    def load_from_h5(self, filename):
        try:
            import h5py
            with h5py.File(filename, "r") as hf:
                data = {k: np.array(hf[k]) for k in hf.keys()}
        except (ImportError, OSError):
            with np.load(filename) as z:
                data = {k: z[k] for k in z.files}
        self.x, self.y, self.z = data["x"], data["y"], data["z"]
        self.Nx, self.Ny, self.Nz = len(self.x) - 1, len(self.y) - 1, len(self.z) - 1
        self.xmin, self.xmax, self.ymin, self.ymax = self.x[0], self.x[-1], self.y[0], self.y[-1]
        self.zmin, self.zmax = self.z[0], self.z[-1]
        self.dx, self.dy, self.dz = np.diff(self.x), np.diff(self.y), np.diff(self.z)
        self._compute_grid()
        self.stl_solids, self.stl_materials, self.stl_colors = {}, {}, {}
        for k, v in data.items():
            if k.startswith("mask:"):
                name = k[5:]
                self.grid[name] = v.astype(bool)
                self.stl_solids[name] = v.astype(bool)
                self.stl_colors[name] = "other"
            elif k.startswith("material:"):
                self.stl_materials[k[9:]] = list(v)
        self.stl_method = "legacy"
        self.use_mesh_refinement = False

    def update_logger(self, attrs):
        for atr in attrs:
            val = getattr(self, atr)
            if atr == "stl_solids" and isinstance(val, dict):
                # solids are masks or callables here, not file names: log what they are
                val = {k: (v if isinstance(v, str) else
                           f"mask{tuple(v.shape)}" if hasattr(v, "shape") else getattr(v, "__name__", type(v).__name__))
                       for k, v in val.items()}
            self.logger.grid[atr] = val
