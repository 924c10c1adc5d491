"""Test-only in-memory stand-in for ``h5py``.

Used solely by ``tests/golden/make_golden.py`` to run the reference Wakis package in a
container where h5py is not installed.  Datasets live in a module-level dict keyed by
absolute file name, so a file written by ``wakesolve`` can be re-opened by
``WakeSolver.read_Ez``.  An empty placeholder is created on disk so that
``os.path.getsize`` works.  Nothing in the product imports this module.
"""

import os

import numpy as np

_STORE = {}


class Dataset:
    def __init__(self, arr):
        self._a = np.asarray(arr)

    @property
    def shape(self):
        return self._a.shape

    @property
    def dtype(self):
        return self._a.dtype

    def __getitem__(self, key):
        return self._a[key]

    def __array__(self, dtype=None, copy=None):
        return self._a if dtype is None else self._a.astype(dtype)

    def __len__(self):
        return len(self._a)


class File:
    def __init__(self, name, mode="r", **kwargs):
        self.filename = os.path.abspath(str(name))
        if mode in ("w", "w-", "x"):
            _STORE[self.filename] = {}
            d = os.path.dirname(self.filename)
            if d:
                os.makedirs(d, exist_ok=True)
            open(self.filename, "wb").close()
        elif self.filename not in _STORE:
            if mode == "a":
                _STORE[self.filename] = {}
            else:
                raise OSError(f"stand-in h5py: no such file {name}")
        self._d = _STORE[self.filename]

    def __setitem__(self, key, value):
        self._d[key] = np.array(value)

    def __getitem__(self, key):
        return Dataset(self._d[key])

    def __contains__(self, key):
        return key in self._d

    def keys(self):
        return list(self._d.keys())

    def create_dataset(self, name, data=None, **kwargs):
        self._d[name] = np.array(data)
        return Dataset(self._d[name])

    def close(self):
        pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False
