"""Test infrastructure only (oracle): ``pyopencl.array`` backed by NumPy arrays in host memory.

Covers the calls made by the reference's UPPE path: ``to_device``, ``empty``, ``zeros``,
``Array.get/set/fill/copy``, slice assignment, ``+``/``*`` between arrays, and the ``sum``,
``max`` and ``min`` reductions (``modules/uppe_kernel.py:64-129,163-185,210,219-223``).
"""
import numpy as np


class Array:
    def __init__(self, ary):
        ary = np.asarray(ary)
        self._a = ary if ary.flags['C_CONTIGUOUS'] else np.array(ary, order='C')

    # the kernel launcher reads the host buffer from here
    @property
    def base_array(self):
        return self._a

    @property
    def data(self):
        return self

    @property
    def shape(self):
        return self._a.shape

    @property
    def dtype(self):
        return self._a.dtype

    @property
    def size(self):
        return self._a.size

    @property
    def ndim(self):
        return self._a.ndim

    def get(self, queue=None, ary=None, **k):
        if ary is not None:
            ary[...] = self._a
            return ary
        return self._a.copy()

    def set(self, ary, queue=None, **k):
        ary = np.asarray(ary)
        if ary.shape != self._a.shape and ary.size == self._a.size:
            ary = ary.reshape(self._a.shape)
        self._a[...] = ary

    def fill(self, value, queue=None, **k):
        self._a[...] = value
        return self

    def copy(self, queue=None, **k):
        return Array(self._a.copy())

    def __getitem__(self, idx):
        return Array(self._a[idx])

    def __setitem__(self, idx, value):
        self._a[idx] = value._a if isinstance(value, Array) else value

    def _other(self, o):
        return o._a if isinstance(o, Array) else o

    def __add__(self, o):
        return Array(self._a + self._other(o))

    __radd__ = __add__

    def __sub__(self, o):
        return Array(self._a - self._other(o))

    def __mul__(self, o):
        return Array(self._a * self._other(o))

    __rmul__ = __mul__

    def __truediv__(self, o):
        return Array(self._a / self._other(o))

    def __neg__(self):
        return Array(-self._a)


def to_device(queue, ary, **k):
    return Array(np.array(ary, copy=True, order="C"))


def empty(queue, shape, dtype, **k):
    return Array(np.empty(shape, dtype=dtype))


def zeros(queue, shape, dtype, **k):
    return Array(np.zeros(shape, dtype=dtype))


def empty_like(a, **k):
    return Array(np.empty_like(a._a))


def zeros_like(a, **k):
    return Array(np.zeros_like(a._a))


def sum(a, queue=None, **k):  # noqa: A001
    return Array(np.array(np.sum(a._a)))


def max(a, queue=None, **k):  # noqa: A001
    return Array(np.array(np.max(a._a)))


def min(a, queue=None, **k):  # noqa: A001
    return Array(np.array(np.min(a._a)))
