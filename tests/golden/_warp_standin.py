"""A pure-Python interpreter for the subset of NVIDIA Warp used by stonewall3d/lbm3d.py.

TEST INFRASTRUCTURE, used only by make_golden.py in a container that has the
reference sources.  Warp (the reference's third-party runtime, version
unpinned, not installable here) is absent, so lbm3d.py cannot be imported as
is.  Installing this module as ``sys.modules["warp"]`` lets the reference's own
kernel bodies (k_init, k_step, k_macro, k_accum, k_slice_*, k_qcoarse) and its
main() driver run unchanged: every kernel thread is executed as a Python call
with float32 numpy scalars (``float`` inside a kernel is rebound to
numpy.float32, as Warp types it), so each arithmetic operation rounds to
float32 in source order.

What is NOT reproduced from Warp: its code generator's FMA contraction on the
GPU, and its random-number stream.  wp.rand_init / wp.randf are restated from
the published PCG hash (Jarzynski & Olano, JCGT 2020) as
state = pcg(seed + pcg(offset)), randf = (pcg(state) >> 8) / 2^24; the product
and the oracle use the same restatement, so their k_init matches these
fixtures, but the stream is not pinned against Warp itself.

wp.atomic_add accumulates in the dtype of the target array, in thread order
(x, y, z): into a float32 array exactly as the reference's float32 atomics
would in that order, into a float64 array to give a reference sum without
float32 accumulation error.
"""
import inspect
import itertools
import types

import numpy as np

float32 = np.float32
float64 = np.float64
uint8 = np.uint8
int32 = np.int32
uint32 = np.uint32

_tid = None


def init():
    return None


def synchronize_device(device=None):
    return None


def _np_dtype(dtype):
    if dtype is None or dtype is float or dtype is np.float32:
        return np.float32
    return np.dtype(dtype).type


class _Annot:
    def __init__(self, ndim, dtype):
        self.ndim, self.dtype = ndim, dtype


class StubArray:
    def __init__(self, a):
        self.a = a

    @property
    def shape(self):
        return self.a.shape

    def numpy(self):
        return self.a.copy()

    def assign(self, other):
        src = other.a if isinstance(other, StubArray) else np.asarray(other)
        self.a[...] = src


def array(data=None, dtype=None, device=None, **kw):
    if data is None:                       # used as a type annotation: wp.array(dtype=float)
        return _Annot(1, dtype)
    return StubArray(np.array(data, dtype=_np_dtype(dtype)))


def array3d(dtype=None):
    return _Annot(3, dtype)


def array4d(dtype=None):
    return _Annot(4, dtype)


def zeros(shape, dtype=float, device=None, **kw):
    return StubArray(np.zeros(shape, dtype=_np_dtype(dtype)))


def vector(length, dtype=float):
    return np.zeros(length, dtype=_np_dtype(dtype))


def tid():
    return _tid


def sqrt(x):
    if type(x) is float:                 # a literal such as wp.sqrt(2.0) is float32 in Warp
        x = np.float32(x)
    return np.sqrt(x)


def max(a, b):  # noqa: A001  (Warp's name)
    return a if a >= b else b


def atomic_add(arr, *args):
    idx, val = args[:-1], args[-1]
    arr[idx] = arr[idx] + val            # float32 + float32 rounds to float32; float64 target stays float64


def _pcg(s):
    s &= 0xFFFFFFFF
    b = (s * 747796405 + 2891336453) & 0xFFFFFFFF
    c = (((b >> ((b >> 28) + 4)) ^ b) * 277803737) & 0xFFFFFFFF
    return ((c >> 22) ^ c) & 0xFFFFFFFF


def rand_init(seed, offset=None):
    if offset is None:
        return [_pcg(int(seed))]
    return [_pcg(int(seed) + _pcg(int(offset) & 0xFFFFFFFF))]


def randf(st):
    st[0] = _pcg(st[0])
    return np.float32(st[0] >> 8) * np.float32(1.0 / 16777216.0)


def _rebind(fn):
    g = dict(fn.__globals__)
    g["float"] = np.float32
    return types.FunctionType(fn.__code__, g, fn.__name__, fn.__defaults__, fn.__closure__)


class Func:
    def __init__(self, fn):
        self.fn = fn
        self._f32 = None

    def __call__(self, *args):
        if self._f32 is None:
            self._f32 = _rebind(self.fn)
        return self._f32(*args)


class Kernel(Func):
    pass


def func(fn):
    return Func(fn)


def kernel(fn=None, **kw):
    if fn is None:
        return lambda f: Kernel(f)
    return Kernel(fn)


def _convert(arg, annot):
    if isinstance(arg, StubArray):
        return arg.a
    if isinstance(arg, np.ndarray):
        return arg
    if annot is float:
        return np.float32(arg)
    if annot is int:
        return int(arg)
    return arg


def launch(k, dim, inputs, device=None, **kw):
    global _tid
    params = list(inspect.signature(k.fn).parameters.values())
    args = [_convert(a, p.annotation) for a, p in zip(inputs, params)]
    if isinstance(dim, int):
        dim = (dim,)
    for t in itertools.product(*[range(d) for d in dim]):
        _tid = t if len(t) > 1 else t[0]
        k(*args)
    _tid = None
