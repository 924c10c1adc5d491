"""Field: a 3-component vector field stored as one flat array of length 3*N.

Same layout and access semantics as the reference's Field (wakis/field.py:19-570):
component blocks [x | y | z], each in Fortran ("lexicographic") order
n = i + Nx*j + Nx*Ny*k; ``toarray()`` returns the flat storage; tuple indexing
``F[i, j, k, 'x'|'y'|'z'|'Abs']`` reads or writes a sub-block.  The storage is a torch
tensor (on the GPU for the solver's E, H, J), so kernels of libwakis_fit read and write
it in place.  Reading a sub-block returns a numpy array (a device->host copy on the GPU,
as the reference's cupy path does with ``.get()``).
"""

import numpy as np
import torch

_NP2T = {
    np.dtype(np.float64): torch.float64,
    np.dtype(np.float32): torch.float32,
    np.dtype(np.int8): torch.int8,
    np.dtype(np.int32): torch.int32,
    np.dtype(np.int64): torch.int64,
    np.dtype(np.bool_): torch.bool,
    np.dtype(np.complex128): torch.complex128,
}


def torch_dtype(dtype):
    if isinstance(dtype, torch.dtype):
        return dtype
    return _NP2T[np.dtype(dtype)]


def _comp_id(key):
    if key == 0 or key == "x":
        return 0
    if key == 1 or key == "y":
        return 1
    if key == 2 or key == "z":
        return 2
    raise IndexError("Component id not valid")


def _index(k, size):
    """torch-compatible index for one axis (numpy semantics: negative ints, any slice)."""
    if isinstance(k, (np.integer,)):
        k = int(k)
    if isinstance(k, slice):
        if k.step is not None and k.step < 0:
            return torch.as_tensor(np.ascontiguousarray(np.arange(size)[k]))
        return k
    if isinstance(k, (list, tuple, np.ndarray)):
        return torch.as_tensor(np.asarray(k))
    return k


class Field:
    def __init__(self, Nx, Ny, Nz, dtype=float, use_ones=False, use_gpu=False, device=None):
        self.Nx, self.Ny, self.Nz = int(Nx), int(Ny), int(Nz)
        self.N = self.Nx * self.Ny * self.Nz
        self.dtype = np.dtype(dtype).type if not isinstance(dtype, torch.dtype) else dtype
        self.on_gpu = bool(use_gpu)
        self.xp = torch
        if device is None:
            device = torch.device("cuda", torch.cuda.current_device()) if use_gpu else torch.device("cpu")
        fill = torch.ones if use_ones else torch.zeros
        self.array = fill(3 * self.N, dtype=torch_dtype(self.dtype), device=device)
        self._on_write = None

    # ------------------------------------------------------------------ write hook
    def _notify(self):
        """Runs the owner's hook BEFORE the storage is modified."""
        if self._on_write is not None:
            self._on_write(self)

    @property
    def device(self):
        return self.array.device

    # ------------------------------------------------------------------ components
    @property
    def field_x(self):
        return self.array[0:self.N]

    @property
    def field_y(self):
        return self.array[self.N:2 * self.N]

    @property
    def field_z(self):
        return self.array[2 * self.N:3 * self.N]

    def _set_comp(self, d, value):
        if len(np.shape(value)) > 1:
            self.from_matrix(value, d)
        else:
            self._notify()
            self.array[d * self.N:(d + 1) * self.N] = self._as_tensor(value)

    @field_x.setter
    def field_x(self, value):
        self._set_comp(0, value)

    @field_y.setter
    def field_y(self, value):
        self._set_comp(1, value)

    @field_z.setter
    def field_z(self, value):
        self._set_comp(2, value)

    def _as_tensor(self, value):
        if isinstance(value, torch.Tensor):
            return value.to(device=self.array.device, dtype=self.array.dtype)
        return torch.as_tensor(np.array(value), dtype=self.array.dtype, device=self.array.device)

    def toarray(self):
        return self.array

    def fromarray(self, array):
        self._notify()
        self.array[:] = self._as_tensor(array).reshape(-1)

    def to_matrix(self, key):
        """(Nx, Ny, Nz) view of one component (Fortran order)."""
        d = _comp_id(key)
        return self.array[d * self.N:(d + 1) * self.N].view(self.Nz, self.Ny, self.Nx).permute(2, 1, 0)

    def from_matrix(self, mat, key):
        d = _comp_id(key)
        self._notify()
        self.to_matrix(d).copy_(self._as_tensor(mat).reshape(self.Nx, self.Ny, self.Nz))

    def to_gpu(self):
        self.array = self.array.to("cuda")
        self.on_gpu = True

    def from_gpu(self):
        self.array = self.array.to("cpu")
        self.on_gpu = False

    def numpy(self):
        return self.array.detach().cpu().numpy()

    # ------------------------------------------------------------------ indexing
    def __getitem__(self, key):
        if type(key) is tuple:
            if len(key) != 4:
                raise IndexError("Need 3 indexes and component to access the field")
            if isinstance(key[3], str) and key[3].lower() == "abs":
                return self.get_abs()[key[0], key[1], key[2]]
            m = self.to_matrix(key[3])
            idx = tuple(_index(k, s) for k, s in zip(key[:3], (self.Nx, self.Ny, self.Nz)))
            v = m[idx]
            out = v.detach().cpu().numpy()
            return out[()] if out.ndim == 0 else out
        if type(key) is int or isinstance(key, np.integer):
            if key <= self.N:
                return self.array[int(key)].item()
            raise IndexError("Lexico-graphic index cannot be higher than product of dimensions")
        if type(key) is slice:
            return self.array[key].detach().cpu().numpy()
        raise ValueError("key must be a 3-tuple or an integer")

    def __setitem__(self, key, value):
        self._notify()
        if type(key) is tuple:
            if len(key) != 4:
                raise IndexError("Need 3 indexes and component to access the field")
            m = self.to_matrix(key[3])
            idx = tuple(_index(k, s) for k, s in zip(key[:3], (self.Nx, self.Ny, self.Nz)))
            m[idx] = self._as_tensor(value)
        elif type(key) is int or isinstance(key, np.integer):
            if key <= self.N:
                self.array[int(key)] = self._as_tensor(value)
            else:
                raise IndexError("Lexico-graphic index cannot be higher than product of dimensions")
        elif type(key) is slice:
            self.array[key] = self._as_tensor(value)
        else:
            raise IndexError("key must be a 3-tuple or an integer")

    # ------------------------------------------------------------------ arithmetic
    def _new(self, dtype=None):
        return Field(self.Nx, self.Ny, self.Nz, dtype=dtype or self.dtype, use_gpu=self.on_gpu,
                     device=self.array.device)

    def _operand(self, other):
        if isinstance(other, Field):
            return other.array
        if isinstance(other, (int, float)):
            return other
        return self._as_tensor(other) if not isinstance(other, torch.Tensor) else other.to(self.array.device)

    def _binary(self, other, op, dtype=None):
        out = self._new(dtype)
        if not isinstance(other, (int, float, Field)) and len(np.shape(other)) > 1:
            o = self._as_tensor(other) if not isinstance(other, torch.Tensor) else other.to(self.array.device)
            for d in range(3):
                out.to_matrix(d).copy_(op(self.to_matrix(d), o))
        else:
            out.array = op(self.array, self._operand(other)).to(out.array.dtype)
        return out

    def __mul__(self, other, dtype=None):
        return self._binary(other, lambda a, b: a * b, dtype)

    __rmul__ = __mul__

    def __add__(self, other, dtype=None):
        return self._binary(other, lambda a, b: a + b, dtype)

    __radd__ = __add__

    def __div__(self, other, dtype=None):
        return self._binary(other, lambda a, b: a / b, dtype)

    __truediv__ = __div__

    def __repr__(self):
        return "x:\n" + repr(self.field_x) + "\ny:\n" + repr(self.field_y) + "\nz:\n" + repr(self.field_z)

    __str__ = __repr__

    def copy(self):
        obj = type(self).__new__(self.__class__)
        obj.__dict__.update(self.__dict__)
        obj.array = self.array.clone()
        obj._on_write = None
        return obj

    def compute_ijk(self, n):
        if n > self.N:
            raise IndexError("Lexico-graphic index cannot be higher than product of dimensions")
        k = n // (self.Nx * self.Ny)
        i = (n - k * self.Nx * self.Ny) % self.Nx
        j = (n - k * self.Nx * self.Ny) // self.Nx
        return i, j, k

    def get_abs(self, as_matrix=True):
        """Magnitude sqrt(x^2 + y^2 + z^2) as a numpy array."""
        if as_matrix:
            a = torch.sqrt(self.to_matrix(0) ** 2 + self.to_matrix(1) ** 2 + self.to_matrix(2) ** 2)
        else:
            a = torch.sqrt(self.field_x ** 2 + self.field_y ** 2 + self.field_z ** 2)
        return a.detach().cpu().numpy()

    def inspect(self, *args, **kwargs):
        raise NotImplementedError("Field.inspect needs matplotlib/pyvista rendering, which this package "
                                  "does not provide")

    inspect3D = inspect
