"""Test-only stand-in for ``pyvista`` (absent in this container).

``GridFIT3D._compute_grid`` builds a ``StructuredGrid`` and later code stores the
per-solid cell masks in it (``grid.grid[key]``).  This stand-in is a dict with that
constructor.  Used only by ``tests/golden/make_golden.py``; masks are injected
analytically because STL voxelisation needs VTK.
"""


class StructuredGrid(dict):
    def __init__(self, X=None, Y=None, Z=None):
        super().__init__()
        self.dimensions = None if X is None else X.shape


def __getattr__(name):
    raise AttributeError(f"pyvista stand-in has no attribute {name!r}")
