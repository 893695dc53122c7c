"""pyJvsip-style FFT objects over the GPU library.

The reference exposes its FFT calls to Python through a SWIG module
(python/vsip/vsip.i:522-525, 630-631, 948-949, 1516-1521) wrapped by the
``FFT`` class of python/pyJvsip/pyJvsip.py:3690-3811 and by view properties
(fftip, ifftip, fftop, ifftop, rcfft, crfft: pyJvsip.py:3107-3262).  This
module gives Python callers the same interface on top of this library's C ABI
through ctypes (no SWIG build):

* ``FFT(t, *args)``: t is one of the sixteen type names of ``FFT.tFft``
  ('ccfftip_f' ... 'crfftmop_d'); args are the arguments of the matching
  ``vsip_<t>_create`` call, given one by one or as one tuple.  ``dft(x)``
  transforms in place, ``dft(x, y)`` out of place, and returns the output
  view; ``vsip``, ``type`` and ``arg`` give the plan handle, the type name and
  the creation arguments.  The plan is destroyed with the object.
* ``Block(t, n)`` (t in 'block_f', 'block_d', 'cblock_f', 'cblock_d') holds n
  elements in a numpy array bound as a VSIPL user block, and ``bind`` makes a
  vector view (offset, stride, length) or a matrix view (offset, col_stride,
  col_length, row_stride, row_length) of it; ``create(t, ...)`` makes a
  dense view of a new block.  Views carry ``type`` ('vview_f', 'cmview_d',
  ...), ``vsip`` and the pyJvsip signal-processing properties.

Blocks stay released (host memory): each transform stages its views to the
GPU and back inside the call, so the numpy arrays hold the results when the
call returns.  Unknown types and mismatched views raise ValueError.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import VSIP_COL, VSIP_ROW, lib

_FFT_KINDS = ("ccfftip", "ccfftop", "rcfftop", "crfftop", "ccfftmip", "ccfftmop", "rcfftmop", "crfftmop")

# per transform kind: (input view kind, output view kind or None for in place,
# number of creation arguments, destroy symbol stem)
_KIND_INFO = {
    "ccfftip": ("cvview", None, 5, "vsip_fft_destroy"),
    "ccfftop": ("cvview", "cvview", 5, "vsip_fft_destroy"),
    "rcfftop": ("vview", "cvview", 4, "vsip_fft_destroy"),
    "crfftop": ("cvview", "vview", 4, "vsip_fft_destroy"),
    "ccfftmip": ("cmview", None, 7, "vsip_fftm_destroy"),
    "ccfftmop": ("cmview", "cmview", 7, "vsip_fftm_destroy"),
    "rcfftmop": ("mview", "cmview", 6, "vsip_fftm_destroy"),
    "crfftmop": ("cmview", "mview", 6, "vsip_fftm_destroy"),
}


def _split_type(t: str):
    if not isinstance(t, str) or "_" not in t:
        raise ValueError("FFT type <:%s:> not recognised" % (t,))
    kind, prec = t.rsplit("_", 1)
    if kind not in _KIND_INFO or prec not in ("f", "d"):
        raise ValueError("FFT type <:%s:> not recognised" % (t,))
    return kind, prec


def _create_argtypes(kind: str, prec: str):
    ct = C.c_float if prec == "f" else C.c_double
    u, i = C.c_ulong, C.c_int
    return {
        "ccfftip": [u, ct, i, C.c_uint, i], "ccfftop": [u, ct, i, C.c_uint, i],
        "rcfftop": [u, ct, C.c_uint, i], "crfftop": [u, ct, C.c_uint, i],
        "ccfftmip": [u, u, ct, i, i, C.c_uint, i], "ccfftmop": [u, u, ct, i, i, C.c_uint, i],
        "rcfftmop": [u, u, ct, i, C.c_uint, i], "crfftmop": [u, u, ct, i, C.c_uint, i],
    }[kind]


class FFT:
    """A VSIPL FFT or multiple-FFT plan, pyJvsip style.

    ``FFT('ccfftmop_f', M, N, scale, dir, major, ntimes, hint)`` and so on:
    the arguments are those of ``vsip_<t>_create``."""

    # vector kinds (f, d), then multiple-FFT kinds (f, d), as pyJvsip lists them
    tFft = [k + "_" + p for ks in (_FFT_KINDS[:4], _FFT_KINDS[4:]) for p in ("f", "d") for k in ks]

    def __init__(self, t, *args):
        kind, prec = _split_type(t)
        l = args[0] if len(args) == 1 and isinstance(args[0], tuple) else args
        need = _KIND_INFO[kind][2]
        if len(l) != need:
            raise ValueError("FFT type %s takes %d creation arguments, got %d" % (t, need, len(l)))
        L = lib()
        f = getattr(L, "vsip_%s_create_%s" % (kind, prec))
        f.restype = C.c_void_p
        f.argtypes = _create_argtypes(kind, prec)
        self._h = None
        h = f(*l)
        if not h:
            code = L.jvsip_gpu_last_error()
            msg = L.jvsip_gpu_last_error_string().decode()
            L.jvsip_gpu_clear_error()
            raise RuntimeError("vsip_%s_create_%s failed: error %d: %s" % (kind, prec, code, msg))
        self._h, self._type, self._arg, self._kind, self._prec = h, t, tuple(l), kind, prec

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                getattr(lib(), "%s_%s" % (_KIND_INFO[self._kind][3], self._prec))(C.c_void_p(h))
            except Exception:
                pass
            self._h = None

    def dft(self, *views):
        """One view: in-place transform; two views: out of place.  Returns the output view."""
        if len(views) not in (1, 2):
            raise ValueError("dft takes one view (in place) or two views (out of place)")
        vin, vout_kind = _KIND_INFO[self._kind][0], _KIND_INFO[self._kind][1]
        want = [vin + "_" + self._prec] + ([] if vout_kind is None else [vout_kind + "_" + self._prec])
        got = [getattr(v, "type", None) for v in views]
        if got != want:
            raise ValueError("FFT %s needs views %s, got %s" % (self._type, want, got))
        L = lib()
        f = getattr(L, "vsip_%s_%s" % (self._kind, self._prec))
        f.restype = None
        f.argtypes = [C.c_void_p] * (1 + len(views))
        f(self._h, *[v.vsip for v in views])
        code = L.jvsip_gpu_last_error()
        if code:
            msg = L.jvsip_gpu_last_error_string().decode()
            L.jvsip_gpu_clear_error()
            raise RuntimeError("vsip_%s_%s failed: error %d: %s" % (self._kind, self._prec, code, msg))
        return views[-1]

    @property
    def vsip(self):
        return self._h

    @property
    def type(self):
        return self._type

    @property
    def arg(self):
        return self._arg


# ---------------------------------------------------------------- blocks and views
_BLOCK_TYPES = {"block_f": (False, np.float32), "block_d": (False, np.float64),
                "cblock_f": (True, np.float32), "cblock_d": (True, np.float64)}


class Block:
    """n elements of a real or complex (interleaved) user block in a numpy array."""

    def __init__(self, t: str, n: int):
        if t not in _BLOCK_TYPES:
            raise ValueError("Block type <:%s:> not recognised" % (t,))
        cplx, dt = _BLOCK_TYPES[t]
        self.type, self.length = t, int(n)
        self.complex, self.dtype = cplx, np.dtype(dt)
        self.prec = "f" if self.dtype == np.float32 else "d"
        self.array = np.zeros(2 * self.length if cplx else self.length, dt)
        L = lib()
        name = ("vsip_cblockbind_" if cplx else "vsip_blockbind_") + self.prec
        f = getattr(L, name)
        self._h = f(self.array.ctypes.data, None, self.length, 0) if cplx else f(self.array.ctypes.data, self.length, 0)
        if not self._h:
            raise MemoryError(name + " failed")

    @property
    def vsip(self):
        return self._h

    def bind(self, *a):
        """(offset, stride, length) -> vector view; (offset, col_stride,
        col_length, row_stride, row_length) -> matrix view."""
        if len(a) == 3:
            return VectorView(self, *a)
        if len(a) == 5:
            return MatrixView(self, *a)
        raise ValueError("bind takes 3 (vector) or 5 (matrix) arguments")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                getattr(lib(), ("vsip_cblockdestroy_" if self.complex else "vsip_blockdestroy_") + self.prec)(h)
            except Exception:
                pass
            self._h = None


class _View:
    _destroy = None  # symbol stem of the view's destroy call

    def _index(self):
        raise NotImplementedError

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                getattr(lib(), self._destroy + self.block.prec)(h)
            except Exception:
                pass
            self._h = None

    @property
    def vsip(self):
        return self._h

    @property
    def values(self) -> np.ndarray:
        """A numpy copy of the view's elements (complex views give complex values)."""
        idx = self._index()
        a = self.block.array
        return a[2 * idx] + 1j * a[2 * idx + 1] if self.block.complex else a[idx].copy()

    def fill(self, value):
        self.set(np.full(self._index().shape, value))
        return self

    def set(self, values):
        idx = self._index()
        a = self.block.array
        v = np.asarray(values)
        if self.block.complex:
            a[2 * idx] = v.real
            a[2 * idx + 1] = np.imag(v) if np.iscomplexobj(v) else 0
        else:
            a[idx] = v
        return self


class VectorView(_View):
    def __init__(self, block, offset, stride, length):
        self.block, self.offset, self.stride, self.length = block, int(offset), int(stride), int(length)
        self.type = ("cvview_" if block.complex else "vview_") + block.prec
        self._destroy = "vsip_cvdestroy_" if block.complex else "vsip_vdestroy_"
        L = lib()
        f = getattr(L, ("vsip_cvbind_" if block.complex else "vsip_vbind_") + block.prec)
        self._h = f(block.vsip, self.offset, self.stride, self.length)
        if not self._h:
            raise MemoryError("vector bind failed")

    def _index(self):
        return self.offset + self.stride * np.arange(self.length)

    @property
    def empty(self):
        return create(self.type, self.length)

    def _plan(self, kind, dir):
        return FFT(kind + "_" + self.block.prec, self.length, 1.0, dir, 0, 0)

    @property
    def fftip(self):
        self._need_complex("fftip")
        self._plan("ccfftip", -1).dft(self)
        return self

    @property
    def ifftip(self):
        self._need_complex("ifftip")
        self._plan("ccfftip", 1).dft(self)
        return self

    @property
    def fftop(self):
        if not self.block.complex:  # real input: imaginary part zero, transformed in place
            return create("cvview_" + self.block.prec, self.length).set(self.values).fftip
        out = self.empty
        self._plan("ccfftop", -1).dft(self, out)
        return out

    @property
    def ifftop(self):
        if not self.block.complex:
            return create("cvview_" + self.block.prec, self.length).set(self.values).ifftip
        out = self.empty
        self._plan("ccfftop", 1).dft(self, out)
        return out

    @property
    def rcfft(self):
        if self.block.complex or self.length % 2:
            raise ValueError("rcfft needs a real view of even length")
        out = create("cvview_" + self.block.prec, self.length // 2 + 1)
        FFT("rcfftop_" + self.block.prec, self.length, 1.0, 1, 0).dft(self, out)
        return out

    @property
    def crfft(self):
        if not self.block.complex:
            raise ValueError("crfft needs a complex view")
        n = 2 * (self.length - 1)
        out = create("vview_" + self.block.prec, n)
        FFT("crfftop_" + self.block.prec, n, 1.0, 1, 0).dft(self, out)
        return out

    def _need_complex(self, what):
        if not self.block.complex:
            raise ValueError("%s needs a complex view, got %s" % (what, self.type))


class MatrixView(_View):
    def __init__(self, block, offset, col_stride, col_length, row_stride, row_length, major="ROW"):
        self.block, self.offset = block, int(offset)
        self.col_stride, self.collength = int(col_stride), int(col_length)
        self.row_stride, self.rowlength = int(row_stride), int(row_length)
        self.major = major
        self.type = ("cmview_" if block.complex else "mview_") + block.prec
        self._destroy = "vsip_cmdestroy_" if block.complex else "vsip_mdestroy_"
        L = lib()
        f = getattr(L, ("vsip_cmbind_" if block.complex else "vsip_mbind_") + block.prec)
        self._h = f(block.vsip, self.offset, self.col_stride, self.collength, self.row_stride, self.rowlength)
        if not self._h:
            raise MemoryError("matrix bind failed")

    def _index(self):
        i = np.arange(self.collength)[:, None]
        j = np.arange(self.rowlength)[None, :]
        return self.offset + i * self.col_stride + j * self.row_stride

    def _with_major(self, m):
        v = MatrixView(self.block, self.offset, self.col_stride, self.collength, self.row_stride, self.rowlength, m)
        return v

    @property
    def ROW(self):
        """The same view, transformed along its rows by the properties below."""
        return self._with_major("ROW")

    @property
    def COL(self):
        """The same view, transformed along its columns by the properties below."""
        return self._with_major("COL")

    @property
    def empty(self):
        return create(self.type, self.collength, self.rowlength)._with_major(self.major)

    def _vmajor(self):
        return VSIP_COL if self.major == "COL" else VSIP_ROW

    def _plan(self, kind, dir):
        return FFT(kind + "_" + self.block.prec, self.collength, self.rowlength, 1.0, dir, self._vmajor(), 0, 0)

    @property
    def fftip(self):
        self._need_complex("fftip")
        self._plan("ccfftmip", -1).dft(self)
        return self

    @property
    def ifftip(self):
        self._need_complex("ifftip")
        self._plan("ccfftmip", 1).dft(self)
        return self

    @property
    def fftop(self):
        if not self.block.complex:
            y = create("cmview_" + self.block.prec, self.collength, self.rowlength).set(self.values)
            return y._with_major(self.major).fftip
        out = self.empty
        self._plan("ccfftmop", -1).dft(self, out)
        return out

    @property
    def ifftop(self):
        if not self.block.complex:
            y = create("cmview_" + self.block.prec, self.collength, self.rowlength).set(self.values)
            return y._with_major(self.major).ifftip
        out = self.empty
        self._plan("ccfftmop", 1).dft(self, out)
        return out

    @property
    def rcfft(self):
        if self.block.complex:
            raise ValueError("rcfft needs a real view")
        p = self.block.prec
        if self.major == "COL":
            if self.collength % 2:
                raise ValueError("rcfft needs an even length along the transform direction")
            m, n = self.collength // 2 + 1, self.rowlength
            out = create("cmview_" + p, m, n)
            FFT("rcfftmop_" + p, self.collength, n, 1.0, VSIP_COL, 1, 0).dft(self, out)
        else:
            if self.rowlength % 2:
                raise ValueError("rcfft needs an even length along the transform direction")
            m, n = self.collength, self.rowlength // 2 + 1
            out = create("cmview_" + p, m, n)
            FFT("rcfftmop_" + p, m, self.rowlength, 1.0, VSIP_ROW, 1, 0).dft(self, out)
        return out._with_major(self.major)

    @property
    def crfft(self):
        if not self.block.complex:
            raise ValueError("crfft needs a complex view")
        p = self.block.prec
        if self.major == "COL":
            m, n = 2 * (self.collength - 1), self.rowlength
            out = create("mview_" + p, m, n)
            FFT("crfftmop_" + p, m, n, 1.0, VSIP_COL, 1, 0).dft(self, out)
        else:
            m, n = self.collength, 2 * (self.rowlength - 1)
            out = create("mview_" + p, m, n)
            FFT("crfftmop_" + p, m, n, 1.0, VSIP_ROW, 1, 0).dft(self, out)
        return out._with_major(self.major)

    def _need_complex(self, what):
        if not self.block.complex:
            raise ValueError("%s needs a complex view, got %s" % (what, self.type))


def create(t: str, *dims):
    """A dense view of a new block: 'vview_f' / 'cvview_d' ... with (length,),
    'mview_f' / 'cmview_d' ... with (col_length, row_length), row-major."""
    if not isinstance(t, str) or "_" not in t:
        raise ValueError("view type <:%s:> not recognised" % (t,))
    kind, prec = t.rsplit("_", 1)
    cplx = kind.startswith("c")
    btype = ("cblock_" if cplx else "block_") + prec
    if kind in ("vview", "cvview") and len(dims) == 1:
        return Block(btype, dims[0]).bind(0, 1, dims[0])
    if kind in ("mview", "cmview") and len(dims) == 2:
        m, n = dims
        return Block(btype, m * n).bind(0, n, m, 1, n)
    raise ValueError("view type <:%s:> with dimensions %s not recognised" % (t, dims))
