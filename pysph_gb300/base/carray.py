"""Host-side typed arrays with the reference's carray interface.

The reference keeps particle data in malloc'd C arrays (base/carray.pyx:
``DoubleArray`` :505, ``LongArray`` :1173, ``IntArray`` :171).  Here particle
properties live on the GPU; these small NumPy-backed classes exist for the
places where the reference API hands arrays to or from the user (neighbour
lists from a locator, index lists for ``remove_particles``).
"""
import numpy as np


class BaseArray:
    dtype = np.float64

    def __init__(self, n=0):
        self._data = np.zeros(int(n), dtype=self.dtype)

    @property
    def length(self):
        return self._data.size

    def __len__(self):
        return self._data.size

    def get_npy_array(self):
        return self._data

    def get_data_ptr(self):
        return self._data.ctypes.data

    def set_data(self, data):
        data = np.asarray(data, dtype=self.dtype)
        if data.size != self._data.size:
            raise ValueError("array size mismatch: %d != %d" % (data.size, self._data.size))
        self._data[:] = data

    def resize(self, n):
        d = np.zeros(int(n), dtype=self.dtype)
        k = min(int(n), self._data.size)
        d[:k] = self._data[:k]
        self._data = d

    def append(self, value):
        self._data = np.append(self._data, np.asarray(value, dtype=self.dtype))

    def extend(self, values):
        self._data = np.concatenate([self._data, np.asarray(values, dtype=self.dtype)])

    def reset(self):
        self._data = self._data[:0].copy()

    def remove(self, index_list, input_sorted=False):
        keep = np.ones(self._data.size, bool)
        keep[np.asarray(index_list, dtype=np.int64)] = False
        self._data = self._data[keep]

    def copy_values(self, indices, dest):
        dest.get_npy_array()[:len(indices)] = self._data[np.asarray(indices, np.int64)]

    def __getitem__(self, i):
        return self._data[i]

    def __setitem__(self, i, v):
        self._data[i] = v

    def __iter__(self):
        return iter(self._data.tolist())

    def __repr__(self):
        return "%s(%s)" % (type(self).__name__, self._data.tolist())


class DoubleArray(BaseArray):
    dtype = np.float64


class FloatArray(BaseArray):
    dtype = np.float32


class LongArray(BaseArray):
    dtype = np.int64


class IntArray(BaseArray):
    dtype = np.int32
