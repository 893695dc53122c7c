"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loads ``oracle/liborc_fftm.so`` (building it with gcc when it is missing or
older than its sources) and exposes the VSIPL fftm semantics over numpy
buffers.  Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py`` import this module; the GPU library never does.

Views follow the VSIPL layout (c_VSIP_src/vsip_cmviewattributes_f.h:47-55):
element (i, j) of a complex view lives at complex index
``off + i*col_stride + j*row_stride`` of its block, interleaved (re, im) pairs
unless the block is split into separate real/imaginary arrays.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liborc_fftm.so")
SOURCES = ["fftm_oracle.c", "fftm_oracle_body.h", "fftm_oracle.h"]

CCOP, CCIP, RCOP, CROP = 0, 1, 2, 3
ROW, COL = 0, 1
FWD, INV = -1, 1


def build(force: bool = False) -> str:
    """Compile the oracle with the host gcc (x86_64 here, aarch64 on the GPU host)."""
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    if not force and os.path.exists(LIB_PATH):
        lib_m = os.path.getmtime(LIB_PATH)
        if all(os.path.getmtime(s) <= lib_m for s in srcs):
            return LIB_PATH
    cmd = ["gcc", "-O2", "-std=c99", "-fPIC", "-ffp-contract=off", "-shared",
           "-o", LIB_PATH + ".tmp", srcs[0], "-lm", "-lpthread"]
    subprocess.check_call(cmd)
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


class _CMV(C.Structure):
    _fields_ = [("re", C.c_void_p), ("im", C.c_void_p), ("cst", C.c_long), ("off", C.c_long),
                ("col_stride", C.c_long), ("row_stride", C.c_long),
                ("col_length", C.c_ulong), ("row_length", C.c_ulong)]


class _RMV(C.Structure):
    _fields_ = [("a", C.c_void_p), ("rst", C.c_long), ("off", C.c_long),
                ("col_stride", C.c_long), ("row_stride", C.c_long),
                ("col_length", C.c_ulong), ("row_length", C.c_ulong)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        for sfx, ct in (("_f", C.c_float), ("_d", C.c_double)):
            f = getattr(_lib, "orc_fftm_create" + sfx)
            f.restype = C.c_void_p
            f.argtypes = [C.c_int, C.c_ulong, C.c_ulong, ct, C.c_int, C.c_int]
            getattr(_lib, "orc_fftm_destroy" + sfx).argtypes = [C.c_void_p]
            getattr(_lib, "orc_ccfftmop" + sfx).argtypes = [C.c_void_p, C.POINTER(_CMV), C.POINTER(_CMV)]
            getattr(_lib, "orc_ccfftmip" + sfx).argtypes = [C.c_void_p, C.POINTER(_CMV)]
            getattr(_lib, "orc_rcfftmop" + sfx).argtypes = [C.c_void_p, C.POINTER(_RMV), C.POINTER(_CMV)]
            getattr(_lib, "orc_crfftmop" + sfx).argtypes = [C.c_void_p, C.POINTER(_CMV), C.POINTER(_RMV)]
            mt = getattr(_lib, "orc_ccfftmop_rows_mt" + sfx)
            mt.restype = C.c_int
            mt.argtypes = [C.c_ulong, C.c_ulong, C.c_int, ct, C.c_void_p, C.c_void_p, C.c_int]
            fl = getattr(_lib, "orc_fill" + sfx)
            fl.argtypes = [C.c_void_p, C.c_ulong, C.c_ulonglong, C.c_int]
        _lib.orc_factor.restype = C.c_ulong
        _lib.orc_factor.argtypes = [C.c_ulong] + [C.POINTER(C.c_ulong)] * 3
        _lib.orc_jofk.restype = C.c_ulong
        _lib.orc_jofk.argtypes = [C.c_ulong, C.POINTER(C.c_ulong), C.POINTER(C.c_ulong), C.c_ulong, C.c_ulong]
    return _lib


def sfx(dtype) -> str:
    return "_f" if np.dtype(dtype) == np.float32 else "_d"


# ---------------------------------------------------------------- inputs
def fill(n: int, seed: int, dist: int, dtype=np.float32) -> np.ndarray:
    """n scalars of the shared seeded stream: dist 0 = U[-1,1), 1 = N(0,1)."""
    out = np.empty(n, dtype=dtype)
    if n:
        getattr(lib(), "orc_fill" + sfx(dtype))(out.ctypes.data, n, seed, dist)
    return out


def factor(N: int):
    pn, p0, pF = (C.c_ulong * 6)(), (C.c_ulong * 6)(), (C.c_ulong * 6)()
    k = lib().orc_factor(N, pn, p0, pF)
    return [(int(p0[i]), int(pn[i]), int(pF[i])) for i in range(k)]


def jofk(N: int):
    pn, p0, pF = (C.c_ulong * 6)(), (C.c_ulong * 6)(), (C.c_ulong * 6)()
    k = lib().orc_factor(N, pn, p0, pF)
    if k == 0:
        return []
    return [int(lib().orc_jofk(i, pn, p0, pF[k - 1], k)) for i in range(N)]


# ---------------------------------------------------------------- views
@dataclass
class CView:
    """Complex matrix view over a block: interleaved `buf` (2*size scalars), or
    split real `buf` / imaginary `im` arrays (size scalars each)."""
    buf: np.ndarray
    off: int
    col_stride: int
    col_length: int
    row_stride: int
    row_length: int
    im: Optional[np.ndarray] = None

    @property
    def split(self) -> bool:
        return self.im is not None

    def _c(self) -> _CMV:
        if self.split:
            return _CMV(self.buf.ctypes.data, self.im.ctypes.data, 1, self.off, self.col_stride,
                        self.row_stride, self.col_length, self.row_length)
        isz = self.buf.itemsize
        return _CMV(self.buf.ctypes.data, self.buf.ctypes.data + isz, 2, self.off,
                    self.col_stride, self.row_stride, self.col_length, self.row_length)

    def index(self) -> np.ndarray:
        i = np.arange(self.col_length)[:, None]
        j = np.arange(self.row_length)[None, :]
        return self.off + i * self.col_stride + j * self.row_stride

    def get(self) -> np.ndarray:
        idx = self.index()
        if self.split:
            return self.buf[idx] + 1j * self.im[idx]
        return self.buf[2 * idx] + 1j * self.buf[2 * idx + 1]

    def set(self, z: np.ndarray) -> None:
        idx = self.index()
        if self.split:
            self.buf[idx] = z.real
            self.im[idx] = z.imag
        else:
            self.buf[2 * idx] = z.real
            self.buf[2 * idx + 1] = z.imag


@dataclass
class RView:
    buf: np.ndarray
    off: int
    col_stride: int
    col_length: int
    row_stride: int
    row_length: int
    rst: int = 1

    def _c(self) -> _RMV:
        return _RMV(self.buf.ctypes.data, self.rst, self.off, self.col_stride, self.row_stride,
                    self.col_length, self.row_length)

    def index(self) -> np.ndarray:
        i = np.arange(self.col_length)[:, None]
        j = np.arange(self.row_length)[None, :]
        return self.rst * (self.off + i * self.col_stride + j * self.row_stride)

    def get(self) -> np.ndarray:
        return self.buf[self.index()]

    def set(self, a: np.ndarray) -> None:
        self.buf[self.index()] = a


def dense_cview(M: int, N: int, dtype=np.float32, major: int = ROW, split: bool = False) -> CView:
    """A VSIPL-created style dense view (vsip_cmcreate_f, c_VSIP_src/vsip_cmcreate_f.c)."""
    if split:
        buf, im = np.zeros(M * N, dtype), np.zeros(M * N, dtype)
    else:
        buf, im = np.zeros(2 * M * N, dtype), None
    if major == ROW:
        return CView(buf, 0, N, M, 1, N, im)
    return CView(buf, 0, 1, M, M, N, im)


def dense_rview(M: int, N: int, dtype=np.float32, major: int = ROW) -> RView:
    buf = np.zeros(M * N, dtype)
    if major == ROW:
        return RView(buf, 0, N, M, 1, N)
    return RView(buf, 0, 1, M, M, N)


# ---------------------------------------------------------------- plans
class Plan:
    def __init__(self, kind: int, M: int, N: int, scale: float = 1.0, dir: int = FWD,
                 major: int = ROW, dtype=np.float32):
        self.kind, self.M, self.N, self.scale, self.dir, self.major = kind, M, N, scale, dir, major
        self.dtype = np.dtype(dtype)
        self.s = sfx(dtype)
        self.h = getattr(lib(), "orc_fftm_create" + self.s)(kind, M, N, scale, dir, major)
        if not self.h:
            raise MemoryError("oracle plan creation failed")

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            getattr(lib(), "orc_fftm_destroy" + self.s)(h)
            self.h = None

    def ccfftmop(self, x: CView, y: CView) -> None:
        getattr(lib(), "orc_ccfftmop" + self.s)(self.h, C.byref(x._c()), C.byref(y._c()))

    def ccfftmip(self, y: CView) -> None:
        getattr(lib(), "orc_ccfftmip" + self.s)(self.h, C.byref(y._c()))

    def rcfftmop(self, x: RView, z: CView) -> None:
        getattr(lib(), "orc_rcfftmop" + self.s)(self.h, C.byref(x._c()), C.byref(z._c()))

    def crfftmop(self, z: CView, x: RView) -> None:
        getattr(lib(), "orc_crfftmop" + self.s)(self.h, C.byref(z._c()), C.byref(x._c()))


def ccfftm_rows_mt(x: np.ndarray, dir: int, scale: float, threads: int) -> np.ndarray:
    """Dense row-major ccfftmop over all rows of the interleaved (rows, 2N)
    array `x`, split across `threads` pthreads with one plan each."""
    rows, two_n = x.shape
    y = np.empty_like(x)
    rc = getattr(lib(), "orc_ccfftmop_rows_mt" + sfx(x.dtype))(
        rows, two_n // 2, dir, scale, x.ctypes.data, y.ctypes.data, threads)
    if rc:
        raise RuntimeError("oracle multi-threaded run failed")
    return y


def komega_f(ts, arr, data: RView, freq: CView, gram: RView, scale) -> None:
    """The k-omega step of the reference's kw example (kw.c:8-26) restated:
    the tapers (c_VSIP_src/vsip_vmmul_f.c, ROW then COL: ts[j]*d, then
    arr[i]*(.)), the fftm oracle's rcfftmop (ROW) and ccfftmip (COL, forward,
    scale 1), then |X|^2 as re*re + im*im (vsip_mcmagsq_f.c), scale*p
    (vsip_smmul_f.c) and p + gram (vsip_madd_f.c), each a float32 operation
    rounded once, as the reference's C does."""
    f32 = np.float32
    Nsens, Nts = data.col_length, data.row_length
    d = data.get().astype(f32)
    d = np.multiply(ts[None, :Nts].astype(f32), d, dtype=f32)
    d = np.multiply(arr[:Nsens, None].astype(f32), d, dtype=f32)
    data.set(d)
    Plan(RCOP, Nsens, Nts, 1.0, FWD, ROW, f32).rcfftmop(data, freq)
    Plan(CCIP, Nsens, Nts // 2 + 1, 1.0, FWD, COL, f32).ccfftmip(freq)
    z = freq.get()
    re, im = z.real.astype(f32), z.imag.astype(f32)
    p = np.add(np.multiply(re, re, dtype=f32), np.multiply(im, im, dtype=f32), dtype=f32)
    p = np.multiply(f32(scale), p, dtype=f32)
    freq.set(p.astype(np.complex64) + 1j * im.astype(np.complex64))
    gram.set(np.add(p, gram.get().astype(f32), dtype=f32))
