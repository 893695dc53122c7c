"""ctypes front end of the unmodified jvsip reference library (TEST
INFRASTRUCTURE ONLY; available only where the reference sources exist).

``oracle/Makefile.ref`` compiles the reference's c_VSIP_src into
``oracle/_ref/libvsip_ref.so``.  This module drives that library through its
own public VSIPL API -- user blocks bound to numpy buffers with
vsip_cblockbind_f / vsip_blockbind_f, admitted, viewed with vsip_cmbind_f /
vsip_mbind_f, transformed, released -- so the oracle restatement and the
golden fixtures can be checked against the reference itself.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from pyoracle import CCIP, CCOP, CROP, RCOP, CView, RView, sfx  # noqa: F401

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "_ref", "libvsip_ref.so")
# the reference checkout (its c_VSIP_src/ is compiled); named only by this variable
REF_SRC = os.environ.get("JVSIP_REFERENCE", "")


def available() -> bool:
    return os.path.exists(LIB_PATH) or (bool(REF_SRC) and os.path.isdir(os.path.join(REF_SRC, "c_VSIP_src")))


def build() -> str:
    if not os.path.exists(LIB_PATH):
        if not REF_SRC:
            raise RuntimeError("oracle/_ref/libvsip_ref.so is not built: set JVSIP_REFERENCE to the jvsip "
                               "reference checkout (the directory holding c_VSIP_src/)")
        subprocess.check_call(["make", "-f", os.path.join(HERE, "Makefile.ref"), "-j8",
                               "REF=" + REF_SRC], cwd=REPO)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build(), mode=C.RTLD_LOCAL)
        L = _lib
        for s, ct in (("_f", C.c_float), ("_d", C.c_double)):
            for name in ("ccfftmop_create", "ccfftmip_create"):
                f = getattr(L, "vsip_" + name + s)
                f.restype = C.c_void_p
                f.argtypes = [C.c_ulong, C.c_ulong, ct, C.c_int, C.c_int, C.c_uint, C.c_int]
            for name in ("rcfftmop_create", "crfftmop_create"):
                f = getattr(L, "vsip_" + name + s)
                f.restype = C.c_void_p
                f.argtypes = [C.c_ulong, C.c_ulong, ct, C.c_int, C.c_uint, C.c_int]
            getattr(L, "vsip_fftm_destroy" + s).argtypes = [C.c_void_p]
            for name, n in (("ccfftmop", 3), ("ccfftmip", 2), ("rcfftmop", 3), ("crfftmop", 3)):
                getattr(L, "vsip_" + name + s).argtypes = [C.c_void_p] * n
            f = getattr(L, "vsip_cblockbind" + s)
            f.restype = C.c_void_p
            f.argtypes = [C.c_void_p, C.c_void_p, C.c_ulong, C.c_int]
            f = getattr(L, "vsip_blockbind" + s)
            f.restype = C.c_void_p
            f.argtypes = [C.c_void_p, C.c_ulong, C.c_int]
            getattr(L, "vsip_cblockadmit" + s).argtypes = [C.c_void_p, C.c_int]
            getattr(L, "vsip_blockadmit" + s).argtypes = [C.c_void_p, C.c_int]
            getattr(L, "vsip_cblockrelease" + s).argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
            f = getattr(L, "vsip_blockrelease" + s)
            f.restype = C.c_void_p
            f.argtypes = [C.c_void_p, C.c_int]
            getattr(L, "vsip_cblockdestroy" + s).argtypes = [C.c_void_p]
            getattr(L, "vsip_blockdestroy" + s).argtypes = [C.c_void_p]
            for name in ("vsip_cmbind", "vsip_mbind"):
                f = getattr(L, name + s)
                f.restype = C.c_void_p
                f.argtypes = [C.c_void_p, C.c_ulong, C.c_long, C.c_ulong, C.c_long, C.c_ulong]
            f = getattr(L, "vsip_cmdestroy" + s)
            f.restype = C.c_void_p
            f.argtypes = [C.c_void_p]
            f = getattr(L, "vsip_mdestroy" + s)
            f.restype = C.c_void_p
            f.argtypes = [C.c_void_p]
            # single-FFT plans and vector views
            for name in ("ccfftop_create", "ccfftip_create"):
                f = getattr(L, "vsip_" + name + s)
                f.restype = C.c_void_p
                f.argtypes = [C.c_ulong, ct, C.c_int, C.c_uint, C.c_int]
            for name in ("rcfftop_create", "crfftop_create"):
                f = getattr(L, "vsip_" + name + s)
                f.restype = C.c_void_p
                f.argtypes = [C.c_ulong, ct, C.c_uint, C.c_int]
            getattr(L, "vsip_fft_destroy" + s).argtypes = [C.c_void_p]
            getattr(L, "vsip_fft_getattr" + s).argtypes = [C.c_void_p, C.c_void_p]
            for name, n in (("ccfftop", 3), ("ccfftip", 2), ("rcfftop", 3), ("crfftop", 3)):
                getattr(L, "vsip_" + name + s).argtypes = [C.c_void_p] * n
            for name in ("vsip_cvbind", "vsip_vbind"):
                f = getattr(L, name + s)
                f.restype = C.c_void_p
                f.argtypes = [C.c_void_p, C.c_ulong, C.c_long, C.c_ulong]
            for name in ("vsip_cvdestroy", "vsip_vdestroy"):
                f = getattr(L, name + s)
                f.restype = C.c_void_p
                f.argtypes = [C.c_void_p]
        # the elementwise calls of the k-omega example (kw.c)
        L.vsip_vmmul_f.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
        L.vsip_mcmagsq_f.argtypes = [C.c_void_p, C.c_void_p]
        L.vsip_smmul_f.argtypes = [C.c_float, C.c_void_p, C.c_void_p]
        L.vsip_madd_f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.vsip_mrealview_f.restype = C.c_void_p
        L.vsip_mrealview_f.argtypes = [C.c_void_p]
        L.vsip_vcreate_hanning_f.restype = C.c_void_p
        L.vsip_vcreate_hanning_f.argtypes = [C.c_ulong, C.c_int]
        L.vsip_vget_f.restype = C.c_float
        L.vsip_vget_f.argtypes = [C.c_void_p, C.c_ulong]
        L.vsip_valldestroy_f.argtypes = [C.c_void_p]
        L.vsip_init(None)
    return _lib


class _Bound:
    """A user block bound to a view's numpy storage, admitted for the call."""

    def __init__(self, v, real: bool, with_view: bool = True):
        L, s = lib(), sfx(v.buf.dtype)
        self.L, self.s, self.real = L, s, real
        self.view = None
        if real:
            self.blk = getattr(L, "vsip_blockbind" + s)(v.buf.ctypes.data, v.buf.size, 0)
            getattr(L, "vsip_blockadmit" + s)(self.blk, 1)
            if with_view:
                self.view = getattr(L, "vsip_mbind" + s)(self.blk, v.off, v.col_stride, v.col_length,
                                                         v.row_stride, v.row_length)
        else:
            if v.split:
                self.blk = getattr(L, "vsip_cblockbind" + s)(v.buf.ctypes.data, v.im.ctypes.data,
                                                             v.buf.size, 0)
            else:
                self.blk = getattr(L, "vsip_cblockbind" + s)(v.buf.ctypes.data, None,
                                                             v.buf.size // 2, 0)
            getattr(L, "vsip_cblockadmit" + s)(self.blk, 1)
            if with_view:
                self.view = getattr(L, "vsip_cmbind" + s)(self.blk, v.off, v.col_stride, v.col_length,
                                                          v.row_stride, v.row_length)

    def close(self):
        L, s = self.L, self.s
        if self.real:
            if self.view:
                getattr(L, "vsip_mdestroy" + s)(self.view)
            getattr(L, "vsip_blockrelease" + s)(self.blk, 1)
            getattr(L, "vsip_blockdestroy" + s)(self.blk)
        else:
            if self.view:
                getattr(L, "vsip_cmdestroy" + s)(self.view)
            a, b = C.c_void_p(), C.c_void_p()
            getattr(L, "vsip_cblockrelease" + s)(self.blk, 1, C.byref(a), C.byref(b))
            getattr(L, "vsip_cblockdestroy" + s)(self.blk)


class RefPlan:
    def __init__(self, kind, M, N, scale=1.0, dir=-1, major=0, dtype=np.float32):
        L = lib()
        self.s = sfx(dtype)
        self.kind = kind
        if kind in (CCOP, CCIP):
            name = "ccfftmop_create" if kind == CCOP else "ccfftmip_create"
            self.h = getattr(L, "vsip_" + name + self.s)(M, N, scale, dir, major, 0, 0)
        else:
            name = "rcfftmop_create" if kind == RCOP else "crfftmop_create"
            self.h = getattr(L, "vsip_" + name + self.s)(M, N, scale, major, 0, 0)
        if not self.h:
            raise MemoryError("reference plan creation failed")

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            getattr(lib(), "vsip_fftm_destroy" + self.s)(h)
            self.h = None

    def _run(self, name, *views):
        bound = []
        same = {}
        for v, real in views:
            key = id(v.buf)
            if key in same and not real:
                # the reference allows x and y on one block: bind it once
                b = same[key]
                view = getattr(lib(), "vsip_cmbind" + self.s)(b.blk, v.off, v.col_stride,
                                                               v.col_length, v.row_stride,
                                                               v.row_length)
                bound.append((b, view, True))
                continue
            b = _Bound(v, real)
            same[key] = b
            bound.append((b, b.view, False))
        getattr(lib(), "vsip_" + name + self.s)(self.h, *[bv for _, bv, _ in bound])
        for b, view, extra in bound:
            if extra:
                getattr(lib(), "vsip_cmdestroy" + self.s)(view)
        for b in same.values():
            b.close()

    def ccfftmop(self, x: CView, y: CView):
        self._run("ccfftmop", (x, False), (y, False))

    def ccfftmip(self, y: CView):
        self._run("ccfftmip", (y, False))

    def rcfftmop(self, x: RView, z: CView):
        self._run("rcfftmop", (x, True), (z, False))

    def crfftmop(self, z: CView, x: RView):
        self._run("crfftmop", (z, False), (x, True))


class RefFFT:
    """A reference single-FFT plan (vsip_{cc,rc,cr}fft{op,ip}_create_*) run on
    one-row views: a view with col_length 1 is bound as the vector of its
    row_length elements row_stride apart.  Views whose buffers are the same
    numpy array are bound on one block (x and y in one block)."""

    def __init__(self, kind, N, scale=1.0, dir=-1, dtype=np.float32):
        L = lib()
        self.s = sfx(dtype)
        self.kind = kind
        if kind in (CCOP, CCIP):
            name = "ccfftop_create" if kind == CCOP else "ccfftip_create"
            self.h = getattr(L, "vsip_" + name + self.s)(N, scale, dir, 0, 0)
        else:
            name = "rcfftop_create" if kind == RCOP else "crfftop_create"
            self.h = getattr(L, "vsip_" + name + self.s)(N, scale, 0, 0)
        if not self.h:
            raise MemoryError("reference plan creation failed")

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            getattr(lib(), "vsip_fft_destroy" + self.s)(h)
            self.h = None

    def _run(self, name, *views):
        L, s = lib(), self.s
        blocks = {}
        vecs = []
        for v, real in views:
            assert v.col_length == 1
            key = id(v.buf)
            if key not in blocks:
                blocks[key] = _Bound(v, real, with_view=False)
            b = blocks[key]
            vecs.append(getattr(L, ("vsip_vbind" if real else "vsip_cvbind") + s)(b.blk, v.off, v.row_stride,
                                                                                 v.row_length))
        getattr(L, "vsip_" + name + s)(self.h, *vecs)
        for (v, real), h in zip(views, vecs):
            getattr(L, ("vsip_vdestroy" if real else "vsip_cvdestroy") + s)(h)
        for b in blocks.values():
            b.close()

    def ccfftop(self, x, y):
        self._run("ccfftop", (x, False), (y, False))

    def ccfftip(self, y):
        self._run("ccfftip", (y, False))

    def rcfftop(self, x, z):
        self._run("rcfftop", (x, True), (z, False))

    def crfftop(self, z, x):
        self._run("crfftop", (z, False), (x, True))


def hanning_f(n: int) -> np.ndarray:
    """The reference's vsip_vcreate_hanning_f(n) values."""
    L = lib()
    v = L.vsip_vcreate_hanning_f(n, 0)
    out = np.array([L.vsip_vget_f(v, i) for i in range(n)], np.float32)
    L.vsip_valldestroy_f(v)
    return out


def komega_f(ts, arr, data, freq, gram, scale):
    """kw.c komega() (examples/komegaExamples/kw_c/kw.c:8-26) through the
    reference library: ts / arr are float32 arrays, data an RView (Nsens x Nts),
    freq a CView (Nsens x Nts/2+1, interleaved), gram an RView; all updated in
    place as the reference leaves them."""
    L = lib()
    Nsens, Nts = data.col_length, data.row_length
    Nfreq = Nts // 2 + 1
    tsb = _Bound(RView(ts, 0, 1, 1, 1, ts.size), True, with_view=False)
    arb = _Bound(RView(arr, 0, 1, 1, 1, arr.size), True, with_view=False)
    vts = L.vsip_vbind_f(tsb.blk, 0, 1, Nts)
    varr = L.vsip_vbind_f(arb.blk, 0, 1, Nsens)
    xb, fb, gb = _Bound(data, True), _Bound(freq, False), _Bound(gram, True)
    rc = L.vsip_rcfftmop_create_f(Nsens, Nts, 1.0, 0, 0, 0)
    cc = L.vsip_ccfftmip_create_f(Nsens, Nfreq, 1.0, -1, 1, 0, 0)
    L.vsip_vmmul_f(vts, xb.view, 0, xb.view)
    L.vsip_vmmul_f(varr, xb.view, 1, xb.view)
    L.vsip_rcfftmop_f(rc, xb.view, fb.view)
    L.vsip_ccfftmip_f(cc, fb.view)
    rm = L.vsip_mrealview_f(fb.view)
    L.vsip_mcmagsq_f(fb.view, rm)
    L.vsip_smmul_f(scale, rm, rm)
    L.vsip_madd_f(rm, gb.view, gb.view)
    L.vsip_mdestroy_f(rm)
    L.vsip_fftm_destroy_f(rc)
    L.vsip_fftm_destroy_f(cc)
    L.vsip_vdestroy_f(vts)
    L.vsip_vdestroy_f(varr)
    for b in (tsb, arb, xb, fb, gb):
        b.close()
