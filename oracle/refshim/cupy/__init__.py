"""numpy-backed stand-in for the part of CuPy the reference uses (test infrastructure).

Arrays are numpy arrays of a subclass that adds ``.get()``; math functions are
numpy's. Device attributes report one SM so the reference sizes a 1-block grid.
"""
import numpy as _np

from . import cuda  # noqa: F401


def _plain_index(idx):
    """Integer 0-d arrays (what element reads return here) as Python ints, so
    that a[i][j] = v with i read from another array writes through a view, as
    the pointer arithmetic of a CuPy-JIT kernel does; numpy would treat a 0-d
    array index as advanced indexing and assign into a copy."""
    if isinstance(idx, _np.ndarray) and idx.ndim == 0 and idx.dtype.kind in "iu":
        return int(idx)
    if isinstance(idx, tuple):
        return tuple(_plain_index(i) for i in idx)
    return idx


class ndarray(_np.ndarray):
    def get(self):
        return _np.asarray(self).copy()

    def __setitem__(self, idx, value):
        _np.ndarray.__setitem__(self, _plain_index(idx), value)

    def __getitem__(self, idx):
        out = _np.ndarray.__getitem__(self, _plain_index(idx))
        if isinstance(out, _np.ndarray):
            return out
        # CuPy indexing yields 0-d device arrays that still carry .get()
        return _np.asarray(out).view(ndarray)

    def tolist(self):
        return _np.ndarray.tolist(_np.asarray(self))


def _wrap(a):
    a = _np.asarray(a)
    if a.ndim == 0:
        return a.view(ndarray)
    return a.view(ndarray)


def array(obj, dtype=None, copy=True):
    return _wrap(_np.array(obj, dtype=dtype, copy=True))


def asarray(obj, dtype=None):
    return _wrap(_np.array(obj, dtype=dtype, copy=True))


def zeros(shape, dtype=float):
    return _wrap(_np.zeros(shape, dtype=dtype))


def empty(shape, dtype=float):
    return _wrap(_np.zeros(shape, dtype=dtype))


def full(shape, fill_value, dtype=None):
    return _wrap(_np.full(shape, fill_value, dtype=dtype))


def concatenate(arrs, axis=0):
    return _wrap(_np.concatenate([_np.asarray(a) for a in arrs], axis=axis))


int8 = _np.int8
int16 = _np.int16
int32 = _np.int32
int64 = _np.int64
uint32 = _np.uint32
uint64 = _np.uint64
float32 = _np.float32
float64 = _np.float64
nan = _np.nan
isnan = _np.isnan
sqrt = _np.sqrt
log = _np.log
cos = _np.cos
sin = _np.sin
exp = _np.exp
floor = _np.floor
abs = _np.abs
