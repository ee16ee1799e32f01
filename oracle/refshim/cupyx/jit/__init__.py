"""Stand-in for cupyx.jit that runs raw kernels as plain Python.

``rawkernel`` returns an object that is callable as a device function and
subscriptable as ``kernel[grid, block](*args)``. Launches run the Python body
once with blockIdx = threadIdx = 0 and gridDim = blockDim = 1, i.e. one thread
executes the whole grid-stride loop, which is the reference kernel's semantics
for a 1x1 launch.
"""
from . import _builtin_funcs, _cuda_types, _internal_types  # noqa: F401


class _Dim3:
    def __init__(self, x):
        self.x = x
        self.y = 0 if x == 0 else 1
        self.z = 0 if x == 0 else 1


blockIdx = _Dim3(0)
threadIdx = _Dim3(0)
blockDim = _Dim3(1)
gridDim = _Dim3(1)


def syncthreads():
    return None


def threadfence():
    return None


def atomic_add(array, index, value):
    old = array[index]
    array[index] = old + value
    return old


class _RawKernel:
    def __init__(self, func, device=False):
        self._func = func
        self.__name__ = getattr(func, "__name__", "rawkernel")
        self.__doc__ = getattr(func, "__doc__", None)
        self.__wrapped__ = func

    def __call__(self, *args):
        return self._func(*args)

    def __getitem__(self, launch):
        grid, block = launch
        if int(grid) < 1 or int(block) < 1:
            raise ValueError("refshim: empty launch")

        def _launch(*args):
            return self._func(*args)

        return _launch


def rawkernel(*, mode="python", device=False):
    def deco(func):
        return _RawKernel(func, device=device)

    return deco
