"""Run the reference's own EFF code on the CPU to make golden vectors.

TEST INFRASTRUCTURE ONLY.  Needs the reference checkout; used by
``tests/golden/make_golden.py`` in the container where fixtures are made,
never on a GPU machine and never by the product.

What runs is the reference itself, not a restatement:

* the Python source of ``OlaGPU.__init__/cnv/cnvtp/fft/deconv``
  (olaGPU.py:95-311, 312-733, 813-824; ``deconv`` is run in its 'xdirect'
  mode), ``window`` and ``win2winaux`` (imagetools.py:314-344, 398-454) and
  the ``gputools`` wrappers on the path (gputools.py:322-401, 498-519,
  546-569, 599-640, 1025-1044, 1068-1181), read from the reference files
  and executed unchanged except for the substitutions below;
* the reference's CUDA kernels (gputools.cu) compiled for the CPU into
  ``oracle/_ref`` by ``oracle/build_ref.py``, launched with the grid and
  block sizes the wrappers compute.

Stand-ins replace what is absent here: PyCUDA's ``gpuarray`` becomes a numpy
subclass whose ``gpudata`` is the host address; ``module_from_buffer`` /
``get_function`` dispatch to the CPU-compiled kernels; pyfft's
``Plan.execute`` is an in-place complex64 ``numpy.fft.fft2`` over the batch
at the given address (so the FFT itself is not the reference's; pyfft 0.3.5
is not available).

Substitutions: (1) ``x == None`` becomes ``x is None`` (2011-era numpy
returned a scalar False for ``array == None``; today's compares elementwise).
(2) ``OlaGPU.cnvtp`` overlap-adds ``sw``-sized slices with extent
``sw + sf - 1`` (olaGPU.py:307), which reads past the end of the slice stack;
the harness passes extent ``sw`` there so that no out-of-bounds memory is
read.
"""
from __future__ import annotations

import ctypes
import os
import re
import types

import numpy as np
from scipy import signal

from . import build_ref

REF_DIR = build_ref.reference_dir()

# --------------------------------------------------------------------------
# PyCUDA / pyfft stand-ins
# --------------------------------------------------------------------------


class GPUArray(np.ndarray):
    """Host array posing as ``pycuda.gpuarray.GPUArray``."""

    @property
    def gpudata(self):
        assert self.flags["C_CONTIGUOUS"]
        return self.ctypes.data

    def get(self):
        return np.array(self)

    @property
    def real(self):
        """PyCUDA's ``.real`` is a new contiguous array."""
        return _wrap(np.real(np.asarray(self)))


def _keep_dtype(name):
    """PyCUDA array-scalar arithmetic keeps the array's dtype (numpy 2 would
    promote e.g. complex64 / int64 to complex128)."""
    base = getattr(np.ndarray, name)

    def op(self, other):
        r = base(self, other)
        if np.ndim(other) == 0 and isinstance(r, np.ndarray) and r.dtype != self.dtype:
            r = r.astype(self.dtype)
        return r
    return op


for _name in ("__add__", "__radd__", "__sub__", "__rsub__", "__mul__", "__rmul__",
              "__truediv__", "__rtruediv__"):
    setattr(GPUArray, _name, _keep_dtype(_name))


def _to_gpu(x):
    return np.ascontiguousarray(x).view(GPUArray)


def _wrap(a):
    return np.ascontiguousarray(a).view(GPUArray)


def _dot(a, b, dtype=None):
    r = np.vdot(np.asarray(a).ravel(), np.asarray(b).ravel())
    return _wrap(np.array(r, dtype=dtype or np.result_type(a, b)))


# ``crop_Kernel`` (gputools.cu:254-263) does not bound its source index: when
# the patch grid covers less than the image, ``crop_gpu2cpu`` reads past the
# end of the overlap-added array.  Allocations carry a NaN-filled tail so those
# reads stay inside host memory and show up as NaN (or as values aliased from
# the next row) instead of faulting; fixtures mask that region.
_TAIL = 1 << 16


def _alloc(shape, dtype, fill):
    shape = tuple(int(v) for v in np.atleast_1d(shape))
    n = int(np.prod(shape))
    buf = np.full(n + _TAIL, np.nan, dtype=dtype)
    buf[:n] = fill
    return buf[:n].reshape(shape).view(GPUArray)


cua = types.SimpleNamespace(
    GPUArray=GPUArray,
    to_gpu=_to_gpu,
    empty=lambda shape, dtype: _alloc(shape, dtype, np.nan),
    zeros=lambda shape, dtype: _alloc(shape, dtype, 0),
    empty_like=lambda a: _alloc(a.shape, a.dtype, np.nan),
    zeros_like=lambda a: _alloc(a.shape, a.dtype, 0),
    dot=_dot,
)

_LIB = None


def _lib():
    global _LIB
    if _LIB is None:
        path = build_ref.build(REF_DIR, quiet=True)
        if path is None:
            raise RuntimeError("reference checkout not present")
        _LIB = ctypes.CDLL(path)
    return _LIB


def _carg(v):
    if isinstance(v, (np.int32,)):
        return ctypes.c_int32(int(v))
    if isinstance(v, (np.uint32,)):
        return ctypes.c_uint32(int(v))
    if isinstance(v, (np.float32,)):
        return ctypes.c_float(float(v))
    if isinstance(v, int):  # gpudata
        return ctypes.c_void_p(v)
    raise TypeError(f"unsupported kernel argument {type(v)}")


class _Function:
    def __init__(self, name):
        self.fn = getattr(_lib(), "ref_" + name)

    def __call__(self, *args, block, grid):
        gx = grid[0]
        gy = grid[1] if len(grid) > 1 else 1
        self.fn(ctypes.c_uint(gx), ctypes.c_uint(gy), ctypes.c_uint(block[0]),
                ctypes.c_uint(block[1]), *[_carg(a) for a in args])


class _Module:
    def get_function(self, name):
        return _Function(name)


cu = types.SimpleNamespace(module_from_buffer=lambda cubin: _Module())


class _Plan:
    """pyfft ``Plan``: in-place forward complex64 2-D FFT of a batch."""

    def __init__(self, shape):
        self.shape = tuple(int(v) for v in shape)

    def execute(self, ptr, batch=1):
        if isinstance(ptr, np.ndarray):  # pyfft also takes the array itself
            ptr = ptr.gpudata
        n = batch * self.shape[0] * self.shape[1]
        buf = (ctypes.c_float * (2 * n)).from_address(int(ptr))
        a = np.frombuffer(buf, dtype=np.complex64).reshape((batch,) + self.shape)
        a[...] = np.fft.fft2(a.astype(np.complex128)).astype(np.complex64)


cufft = types.SimpleNamespace(Plan=_Plan)


class _Elementwise:
    """``ElementwiseKernel`` for the two clip kernels used on the path."""

    def __init__(self, arguments, operation, name):
        self.name = name

    def __call__(self, x, v):
        if self.name == "cliplower":
            np.maximum(x, np.float32(v), out=x)
        elif self.name == "clipupper":
            np.minimum(x, np.float32(v), out=x)
        else:
            raise NotImplementedError(self.name)


cuelement = types.SimpleNamespace(ElementwiseKernel=_Elementwise)

# 2011-era scipy accepted a float window length (the reference passes the
# float patch size from np.ceil); today's scipy needs an int.
signal_compat = types.SimpleNamespace(
    get_window=lambda name, n, **kw: signal.get_window(name, int(n), **kw))

# --------------------------------------------------------------------------
# Extract and execute the reference's Python
# --------------------------------------------------------------------------


def _source_lines(fname):
    with open(os.path.join(REF_DIR, fname)) as fh:
        return fh.read().split("\n")


def _top_level_block(lines, name):
    """Source of the top-level ``def``/``class`` called ``name``."""
    start = next(i for i, l in enumerate(lines) if re.match(rf"(def|class) {name}\b", l))
    end = start + 1
    while end < len(lines) and (lines[end].strip() == "" or lines[end][0] in " \t#"):
        end += 1
    return "\n".join(lines[start:end])


def _method_block(lines, name):
    """Source of the method ``name`` (4-space indented ``def``)."""
    start = next(i for i, l in enumerate(lines) if re.match(rf"    def {name}\b", l))
    end = start + 1
    while end < len(lines):
        l = lines[end]
        if l.strip() and not l.lstrip().startswith("#") and re.match(r"( {0,4})\S", l):
            break
        end += 1
    return "\n".join(lines[start:end])


def _era_compat(src):
    return src.replace("== None", "is None")


def _module(name, namespace):
    mod = types.ModuleType(name)
    mod.__dict__.update(namespace)
    return mod


def load():
    """Return ``(gputools, imagetools, olaGPU)`` module objects built from the
    reference's source."""
    gt_lines = _source_lines("gputools.py")
    gputools = _module("gputools", {"np": np, "cua": cua, "cu": cu, "cuelement": cuelement,
                                    "cubin": None})
    for fn in ("chop_mod_pad_GPU", "chop_pad_GPU", "crop_gpu2cpu", "crop_stack_GPU",
               "normalize", "ola_GPU_test", "pad_cpu2gpu", "pad_stack_GPU",
               "cliplower_GPU", "clipupper_GPU", "comp_ola_deconv"):
        exec(compile(_era_compat(_top_level_block(gt_lines, fn)), f"gputools.py:{fn}", "exec"),
             gputools.__dict__)

    it_lines = _source_lines("imagetools.py")
    imagetools = _module("imagetools", {"np": np, "signal": signal_compat, "cua": cua,
                                        "gputools": gputools})
    for fn in ("window", "win2winaux"):
        exec(compile(_era_compat(_top_level_block(it_lines, fn)), f"imagetools.py:{fn}", "exec"),
             imagetools.__dict__)

    ola_lines = _source_lines("olaGPU.py")
    methods = {m: _method_block(ola_lines, m) for m in ("__init__", "cnv", "cnvtp", "fft", "deconv")}
    bad = "self.winaux.sw+self.sf-1,"
    assert methods["cnvtp"].count(bad) == 1, "cnvtp overlap-add extent not found"
    methods["cnvtp"] = methods["cnvtp"].replace(bad, "self.winaux.sw,")
    src = "class OlaGPU:\n" + "\n".join(methods[m] for m in ("__init__", "cnv", "cnvtp", "fft", "deconv"))
    olaGPU = _module("olaGPU", {"np": np, "cua": cua, "cufft": cufft, "gputools": gputools})
    exec(compile(_era_compat(src), "olaGPU.py:OlaGPU", "exec"), olaGPU.__dict__)
    return gputools, imagetools, olaGPU
