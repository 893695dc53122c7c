"""jvsip_gb300 -- GB300 (sm_103a) implementation of the VSIPL multiple-FFT
calls and of the single-FFT calls built on them.

The product is the C-ABI shared library ``libjvsip_fftm_gb300.so`` (declared
in ``include/vsip_fftm_gb300.h``).  This package builds it and gives Python
callers (tests, benchmarks, tools) ctypes access to exactly that C API -- the
same function names and argument meanings as the jvsip reference
(c_VSIP_src/vsip.h) -- plus small helpers to bind numpy / pinned buffers to
VSIPL blocks.  There is no Python or CPU implementation of the transforms:
when the library or a GPU is missing the calls fail.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = _build.LIB

VSIP_ROW, VSIP_COL = 0, 1
VSIP_FFT_FWD, VSIP_FFT_INV = -1, 1
VSIP_MEM_NONE = 0
VSIP_ALG_SPACE, VSIP_ALG_TIME, VSIP_ALG_NOISE = 0, 1, 2
JVSIP_FORM_AUTO, JVSIP_FORM_PLAIN, JVSIP_FORM_SPLIT_BF16, JVSIP_FORM_SPLIT_FP16 = 0, 1, 2, 3
JVSIP_FORM_DF64 = 4

# every symbol include/vsip_fftm_gb300.h declares
EXPORTS = [
    "vsip_ccfftmop_create_f", "vsip_ccfftmip_create_f", "vsip_rcfftmop_create_f", "vsip_crfftmop_create_f",
    "vsip_ccfftmop_create_d", "vsip_ccfftmip_create_d", "vsip_rcfftmop_create_d", "vsip_crfftmop_create_d",
    "vsip_fftm_destroy_f", "vsip_fftm_destroy_d", "vsip_fftm_getattr_f", "vsip_fftm_getattr_d",
    "vsip_ccfftmop_f", "vsip_ccfftmip_f", "vsip_rcfftmop_f", "vsip_crfftmop_f",
    "vsip_ccfftmop_d", "vsip_ccfftmip_d", "vsip_rcfftmop_d", "vsip_crfftmop_d",
    "vsip_init", "vsip_finalize",
    "vsip_cblockbind_f", "vsip_cblockbind_d", "vsip_cblockcreate_f", "vsip_cblockcreate_d",
    "vsip_cblockadmit_f", "vsip_cblockadmit_d", "vsip_cblockrelease_f", "vsip_cblockrelease_d",
    "vsip_cblockdestroy_f", "vsip_cblockdestroy_d",
    "vsip_blockbind_f", "vsip_blockbind_d", "vsip_blockcreate_f", "vsip_blockcreate_d",
    "vsip_blockadmit_f", "vsip_blockadmit_d", "vsip_blockrelease_f", "vsip_blockrelease_d",
    "vsip_blockdestroy_f", "vsip_blockdestroy_d",
    "vsip_cmbind_f", "vsip_cmbind_d", "vsip_mbind_f", "vsip_mbind_d",
    "vsip_cmcreate_f", "vsip_cmcreate_d", "vsip_mcreate_f", "vsip_mcreate_d",
    "vsip_cmdestroy_f", "vsip_cmdestroy_d", "vsip_mdestroy_f", "vsip_mdestroy_d",
    "vsip_cmalldestroy_f", "vsip_cmalldestroy_d", "vsip_malldestroy_f", "vsip_malldestroy_d",
    "jvsip_gpu_last_error", "jvsip_gpu_last_error_string", "jvsip_gpu_clear_error",
    "jvsip_cblocksync_f", "jvsip_cblocksync_d", "jvsip_blocksync_f", "jvsip_blocksync_d",
    "jvsip_fftm_setform_f", "jvsip_fftm_getform_f",
    "jvsip_fftm_batch_f", "jvsip_fftm_batch_create_f", "jvsip_fftm_batch_run_f", "jvsip_fftm_batch_destroy_f",
    "jvsip_gpu_build_info", "jvsip_gpu_synchronize", "jvsip_gpu_stream", "jvsip_fftm_passes", "jvsip_fftm_jofk", "jvsip_fftm_graphs",
    "jvsip_gpu_kernel_launches", "jvsip_ccfftm_noalloc_f", "jvsip_fftm_autotune_f",
    "jvsip_fftm_autotune_entries",
    "vsip_ccfftop_create_f", "vsip_ccfftip_create_f", "vsip_rcfftop_create_f", "vsip_crfftop_create_f",
    "vsip_ccfftop_create_d", "vsip_ccfftip_create_d", "vsip_rcfftop_create_d", "vsip_crfftop_create_d",
    "vsip_fft_destroy_f", "vsip_fft_destroy_d", "vsip_fft_getattr_f", "vsip_fft_getattr_d",
    "vsip_ccfftop_f", "vsip_ccfftip_f", "vsip_rcfftop_f", "vsip_crfftop_f",
    "vsip_ccfftop_d", "vsip_ccfftip_d", "vsip_rcfftop_d", "vsip_crfftop_d",
    "vsip_cvbind_f", "vsip_cvbind_d", "vsip_vbind_f", "vsip_vbind_d",
    "vsip_cvcreate_f", "vsip_cvcreate_d", "vsip_vcreate_f", "vsip_vcreate_d",
    "vsip_cvdestroy_f", "vsip_cvdestroy_d", "vsip_vdestroy_f", "vsip_vdestroy_d",
    "vsip_cvalldestroy_f", "vsip_cvalldestroy_d", "vsip_valldestroy_f", "vsip_valldestroy_d",
    "jvsip_komega_f", "jvsip_fftm_setform_d", "jvsip_fftm_getform_d", "jvsip_fftm_loop_f",
    "jvsip_fftm_autotune_plain_f", "jvsip_fftm_autotune_plain_entry_f", "jvsip_gpu_test_wait_expiry",
]


class ScalarMI(C.Structure):
    _fields_ = [("r", C.c_ulong), ("c", C.c_ulong)]


class FftmAttrF(C.Structure):
    _fields_ = [("input", ScalarMI), ("output", ScalarMI), ("place", C.c_int), ("scale", C.c_float),
                ("dir", C.c_int), ("major", C.c_int)]


class FftmAttrD(C.Structure):
    _fields_ = [("input", ScalarMI), ("output", ScalarMI), ("place", C.c_int), ("scale", C.c_double),
                ("dir", C.c_int), ("major", C.c_int)]


class FftAttrF(C.Structure):
    _fields_ = [("input", C.c_ulong), ("output", C.c_ulong), ("place", C.c_int), ("scale", C.c_float),
                ("dir", C.c_int)]


class FftAttrD(C.Structure):
    _fields_ = [("input", C.c_ulong), ("output", C.c_ulong), ("place", C.c_int), ("scale", C.c_double),
                ("dir", C.c_int)]


_lib = None


def build(force: bool = False) -> str:
    return _build.build(force=force)


def lib(load_only: bool = False):
    """The loaded library with argument types set.  Builds it when missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not load_only:
        build()
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("GPU fftm library not built: %s" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    for s, ct in (("_f", C.c_float), ("_d", C.c_double)):
        for name in ("ccfftmop_create", "ccfftmip_create"):
            f = getattr(L, "vsip_" + name + s)
            f.restype = vp
            f.argtypes = [C.c_ulong, C.c_ulong, ct, C.c_int, C.c_int, C.c_uint, C.c_int]
        for name in ("rcfftmop_create", "crfftmop_create"):
            f = getattr(L, "vsip_" + name + s)
            f.restype = vp
            f.argtypes = [C.c_ulong, C.c_ulong, ct, C.c_int, C.c_uint, C.c_int]
        getattr(L, "vsip_fftm_destroy" + s).argtypes = [vp]
        getattr(L, "vsip_fftm_getattr" + s).argtypes = [vp, vp]
        for name, n in (("ccfftmop", 3), ("ccfftmip", 2), ("rcfftmop", 3), ("crfftmop", 3)):
            getattr(L, "vsip_" + name + s).argtypes = [vp] * n
            getattr(L, "vsip_" + name + s).restype = None
        f = getattr(L, "vsip_cblockbind" + s)
        f.restype = vp
        f.argtypes = [vp, vp, C.c_ulong, C.c_int]
        f = getattr(L, "vsip_cblockcreate" + s)
        f.restype = vp
        f.argtypes = [C.c_ulong, C.c_int]
        f = getattr(L, "vsip_blockbind" + s)
        f.restype = vp
        f.argtypes = [vp, C.c_ulong, C.c_int]
        f = getattr(L, "vsip_blockcreate" + s)
        f.restype = vp
        f.argtypes = [C.c_ulong, C.c_int]
        getattr(L, "vsip_cblockadmit" + s).argtypes = [vp, C.c_int]
        getattr(L, "vsip_blockadmit" + s).argtypes = [vp, C.c_int]
        getattr(L, "vsip_cblockrelease" + s).argtypes = [vp, C.c_int, vp, vp]
        f = getattr(L, "vsip_blockrelease" + s)
        f.restype = vp
        f.argtypes = [vp, C.c_int]
        getattr(L, "vsip_cblockdestroy" + s).argtypes = [vp]
        getattr(L, "vsip_blockdestroy" + s).argtypes = [vp]
        for name in ("vsip_cmbind", "vsip_mbind"):
            f = getattr(L, name + s)
            f.restype = vp
            f.argtypes = [vp, C.c_ulong, C.c_long, C.c_ulong, C.c_long, C.c_ulong]
        for name in ("vsip_cmcreate", "vsip_mcreate"):
            f = getattr(L, name + s)
            f.restype = vp
            f.argtypes = [C.c_ulong, C.c_ulong, C.c_int, C.c_int]
        for name in ("vsip_cmdestroy", "vsip_mdestroy"):
            f = getattr(L, name + s)
            f.restype = vp
            f.argtypes = [vp]
        getattr(L, "vsip_cmalldestroy" + s).argtypes = [vp]
        getattr(L, "vsip_malldestroy" + s).argtypes = [vp]
        for name in ("ccfftop_create", "ccfftip_create"):
            f = getattr(L, "vsip_" + name + s)
            f.restype = vp
            f.argtypes = [C.c_ulong, ct, C.c_int, C.c_uint, C.c_int]
        for name in ("rcfftop_create", "crfftop_create"):
            f = getattr(L, "vsip_" + name + s)
            f.restype = vp
            f.argtypes = [C.c_ulong, ct, C.c_uint, C.c_int]
        getattr(L, "vsip_fft_destroy" + s).argtypes = [vp]
        getattr(L, "vsip_fft_getattr" + s).argtypes = [vp, vp]
        for name, n in (("ccfftop", 3), ("ccfftip", 2), ("rcfftop", 3), ("crfftop", 3)):
            getattr(L, "vsip_" + name + s).argtypes = [vp] * n
            getattr(L, "vsip_" + name + s).restype = None
        for name in ("vsip_cvbind", "vsip_vbind"):
            f = getattr(L, name + s)
            f.restype = vp
            f.argtypes = [vp, C.c_ulong, C.c_long, C.c_ulong]
        for name in ("vsip_cvcreate", "vsip_vcreate"):
            f = getattr(L, name + s)
            f.restype = vp
            f.argtypes = [C.c_ulong, C.c_int]
        for name in ("vsip_cvdestroy", "vsip_vdestroy"):
            f = getattr(L, name + s)
            f.restype = vp
            f.argtypes = [vp]
        getattr(L, "vsip_cvalldestroy" + s).argtypes = [vp]
        getattr(L, "vsip_valldestroy" + s).argtypes = [vp]
        getattr(L, "jvsip_cblocksync" + s).argtypes = [vp]
        getattr(L, "jvsip_blocksync" + s).argtypes = [vp]
    L.jvsip_gpu_last_error_string.restype = C.c_char_p
    L.jvsip_gpu_build_info.restype = C.c_char_p
    L.jvsip_gpu_stream.restype = vp
    L.jvsip_gpu_kernel_launches.restype = C.c_ulong
    L.jvsip_gpu_test_wait_expiry.argtypes = [C.c_int]
    L.jvsip_ccfftm_noalloc_f.argtypes = [vp, vp, C.c_long, vp, C.c_long]
    L.jvsip_fftm_autotune_f.argtypes = [C.c_size_t, vp, C.c_int]
    L.jvsip_fftm_autotune_entries.restype = C.c_long
    L.jvsip_fftm_autotune_plain_f.argtypes = [C.c_size_t, vp, C.c_int]
    ip = C.POINTER(C.c_int)
    L.jvsip_fftm_autotune_plain_entry_f.argtypes = [C.c_ulong, C.c_int, ip, ip, ip, ip, C.c_int]
    L.jvsip_fftm_setform_f.argtypes = [vp, C.c_int]
    L.jvsip_fftm_getform_f.argtypes = [vp]
    L.jvsip_fftm_setform_d.argtypes = [vp, C.c_int]
    L.jvsip_fftm_getform_d.argtypes = [vp]
    L.jvsip_fftm_batch_f.argtypes = [C.c_size_t, vp, vp, vp]
    L.jvsip_fftm_batch_create_f.restype = vp
    L.jvsip_fftm_batch_create_f.argtypes = [C.c_size_t, vp, vp, vp]
    L.jvsip_fftm_batch_run_f.argtypes = [vp]
    L.jvsip_fftm_batch_destroy_f.argtypes = [vp]
    L.jvsip_fftm_loop_f.argtypes = [C.c_size_t, vp, vp, vp]
    L.jvsip_fftm_passes.argtypes = [vp, C.POINTER(C.c_int), C.c_int]
    L.jvsip_fftm_graphs.argtypes = [vp]
    L.jvsip_fftm_graphs.restype = C.c_int
    L.jvsip_komega_f.argtypes = [vp, vp, vp, vp, vp, vp, C.c_float, vp]
    L.jvsip_fftm_jofk.restype = C.c_long
    L.jvsip_fftm_jofk.argtypes = [vp, C.POINTER(C.c_ulong), C.c_long]
    _lib = L
    return L


def sfx(dtype) -> str:
    return "_f" if np.dtype(dtype) == np.float32 else "_d"


def last_error():
    L = lib()
    return int(L.jvsip_gpu_last_error()), L.jvsip_gpu_last_error_string().decode()


def check(what: str = "call"):
    code, msg = last_error()
    if code:
        lib().jvsip_gpu_clear_error()
        raise RuntimeError("%s failed: error %d: %s" % (what, code, msg))


# ---------------------------------------------------------------------------- host helpers
class CBlock:
    """A complex user block bound to numpy storage (interleaved: one array of
    2*n scalars; split: `re` and `im` arrays of n scalars)."""

    def __init__(self, re: np.ndarray, im: np.ndarray | None = None, admit: bool = False, update: bool = True):
        self.s = sfx(re.dtype)
        self.re, self.im = re, im
        n = re.size if im is not None else re.size // 2
        L = lib()
        self.h = getattr(L, "vsip_cblockbind" + self.s)(re.ctypes.data, None if im is None else im.ctypes.data,
                                                        n, 0)
        if not self.h:
            raise MemoryError("vsip_cblockbind failed")
        self.admitted = False
        if admit:
            self.admit(update)

    def admit(self, update: bool = True):
        rc = getattr(lib(), "vsip_cblockadmit" + self.s)(self.h, 1 if update else 0)
        if rc:
            raise RuntimeError("vsip_cblockadmit failed")
        self.admitted = True

    def release(self, update: bool = True):
        a, b = C.c_void_p(), C.c_void_p()
        getattr(lib(), "vsip_cblockrelease" + self.s)(self.h, 1 if update else 0, C.byref(a), C.byref(b))
        self.admitted = False

    def sync(self):
        return getattr(lib(), "jvsip_cblocksync" + self.s)(self.h)

    def destroy(self):
        if self.h:
            getattr(lib(), "vsip_cblockdestroy" + self.s)(self.h)
            self.h = None

    def view(self, off, col_stride, col_length, row_stride, row_length):
        return CMView(self, off, col_stride, col_length, row_stride, row_length)

    def vview(self, off, stride, length):
        return CVView(self, off, stride, length)


class RBlock:
    def __init__(self, a: np.ndarray, admit: bool = False, update: bool = True):
        self.s = sfx(a.dtype)
        self.a = a
        L = lib()
        self.h = getattr(L, "vsip_blockbind" + self.s)(a.ctypes.data, a.size, 0)
        if not self.h:
            raise MemoryError("vsip_blockbind failed")
        if admit:
            self.admit(update)

    def admit(self, update: bool = True):
        if getattr(lib(), "vsip_blockadmit" + self.s)(self.h, 1 if update else 0):
            raise RuntimeError("vsip_blockadmit failed")

    def release(self, update: bool = True):
        getattr(lib(), "vsip_blockrelease" + self.s)(self.h, 1 if update else 0)

    def sync(self):
        return getattr(lib(), "jvsip_blocksync" + self.s)(self.h)

    def destroy(self):
        if self.h:
            getattr(lib(), "vsip_blockdestroy" + self.s)(self.h)
            self.h = None

    def view(self, off, col_stride, col_length, row_stride, row_length):
        return MView(self, off, col_stride, col_length, row_stride, row_length)

    def vview(self, off, stride, length):
        return VView(self, off, stride, length)


class CMView:
    def __init__(self, blk, off, cs, cl, rs, rl):
        self.blk = blk
        self.h = getattr(lib(), "vsip_cmbind" + blk.s)(blk.h, off, cs, cl, rs, rl)

    def destroy(self):
        if self.h:
            getattr(lib(), "vsip_cmdestroy" + self.blk.s)(self.h)
            self.h = None


class MView:
    def __init__(self, blk, off, cs, cl, rs, rl):
        self.blk = blk
        self.h = getattr(lib(), "vsip_mbind" + blk.s)(blk.h, off, cs, cl, rs, rl)

    def destroy(self):
        if self.h:
            getattr(lib(), "vsip_mdestroy" + self.blk.s)(self.h)
            self.h = None


class CVView:
    def __init__(self, blk, off, stride, length):
        self.blk = blk
        self.h = getattr(lib(), "vsip_cvbind" + blk.s)(blk.h, off, stride, length)

    def destroy(self):
        if self.h:
            getattr(lib(), "vsip_cvdestroy" + self.blk.s)(self.h)
            self.h = None


class VView:
    def __init__(self, blk, off, stride, length):
        self.blk = blk
        self.h = getattr(lib(), "vsip_vbind" + blk.s)(blk.h, off, stride, length)

    def destroy(self):
        if self.h:
            getattr(lib(), "vsip_vdestroy" + self.blk.s)(self.h)
            self.h = None


KIND_CCOP, KIND_CCIP, KIND_RCOP, KIND_CROP = 0, 1, 2, 3


class FFTM:
    """A vsip_fftm_{f,d} plan (create / run / getattr / destroy)."""

    def __init__(self, kind: int, M: int, N: int, scale: float = 1.0, dir: int = VSIP_FFT_FWD,
                 major: int = VSIP_ROW, dtype=np.float32, ntimes: int = 0, hint: int = VSIP_ALG_TIME):
        self.kind, self.s = kind, sfx(dtype)
        L = lib()
        if kind in (KIND_CCOP, KIND_CCIP):
            name = "vsip_ccfftmop_create" if kind == KIND_CCOP else "vsip_ccfftmip_create"
            self.h = getattr(L, name + self.s)(M, N, scale, dir, major, ntimes, hint)
        else:
            name = "vsip_rcfftmop_create" if kind == KIND_RCOP else "vsip_crfftmop_create"
            self.h = getattr(L, name + self.s)(M, N, scale, major, ntimes, hint)
        if not self.h:
            check("plan create")
            raise RuntimeError("plan create failed")

    def destroy(self):
        if self.h:
            getattr(lib(), "vsip_fftm_destroy" + self.s)(self.h)
            self.h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    def getattr(self):
        a = FftmAttrF() if self.s == "_f" else FftmAttrD()
        getattr(lib(), "vsip_fftm_getattr" + self.s)(self.h, C.byref(a))
        return a

    def setform(self, form: int):
        rc = getattr(lib(), "jvsip_fftm_setform" + self.s)(self.h, form)
        if rc:
            raise RuntimeError("jvsip_fftm_setform%s failed: %d" % (self.s, rc))

    def passes(self):
        buf = (C.c_int * 40)()
        n = lib().jvsip_fftm_passes(self.h, buf, 40)
        return list(buf[:n])

    def jofk(self, n):
        buf = (C.c_ulong * n)()
        m = lib().jvsip_fftm_jofk(self.h, buf, n)
        return [int(v) for v in buf[:m]]

    def ccfftmop(self, x: CMView, y: CMView):
        getattr(lib(), "vsip_ccfftmop" + self.s)(self.h, x.h, y.h)
        check("vsip_ccfftmop")

    def ccfftmip(self, x: CMView):
        getattr(lib(), "vsip_ccfftmip" + self.s)(self.h, x.h)
        check("vsip_ccfftmip")

    def rcfftmop(self, x: MView, z: CMView):
        getattr(lib(), "vsip_rcfftmop" + self.s)(self.h, x.h, z.h)
        check("vsip_rcfftmop")

    def crfftmop(self, z: CMView, x: MView):
        getattr(lib(), "vsip_crfftmop" + self.s)(self.h, z.h, x.h)
        check("vsip_crfftmop")


class FFT:
    """A vsip_fft_{f,d} single-FFT plan (create / run / getattr / destroy).
    N is the transform length (the real length for rcfftop / crfftop)."""

    def __init__(self, kind: int, N: int, scale: float = 1.0, dir: int = VSIP_FFT_FWD, dtype=np.float32,
                 ntimes: int = 0, hint: int = VSIP_ALG_TIME):
        self.kind, self.s = kind, sfx(dtype)
        L = lib()
        if kind in (KIND_CCOP, KIND_CCIP):
            name = "vsip_ccfftop_create" if kind == KIND_CCOP else "vsip_ccfftip_create"
            self.h = getattr(L, name + self.s)(N, scale, dir, ntimes, hint)
        else:
            name = "vsip_rcfftop_create" if kind == KIND_RCOP else "vsip_crfftop_create"
            self.h = getattr(L, name + self.s)(N, scale, ntimes, hint)
        if not self.h:
            check("plan create")
            raise RuntimeError("plan create failed")

    def destroy(self):
        if self.h:
            getattr(lib(), "vsip_fft_destroy" + self.s)(self.h)
            self.h = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    def getattr(self):
        a = FftAttrF() if self.s == "_f" else FftAttrD()
        getattr(lib(), "vsip_fft_getattr" + self.s)(self.h, C.byref(a))
        return a

    def passes(self):
        buf = (C.c_int * 40)()
        n = lib().jvsip_fftm_passes(self.h, buf, 40)
        return list(buf[:n])

    def ccfftop(self, x: CVView, y: CVView):
        getattr(lib(), "vsip_ccfftop" + self.s)(self.h, x.h, y.h)
        check("vsip_ccfftop")

    def ccfftip(self, x: CVView):
        getattr(lib(), "vsip_ccfftip" + self.s)(self.h, x.h)
        check("vsip_ccfftip")

    def rcfftop(self, x: VView, z: CVView):
        getattr(lib(), "vsip_rcfftop" + self.s)(self.h, x.h, z.h)
        check("vsip_rcfftop")

    def crfftop(self, z: CVView, x: VView):
        getattr(lib(), "vsip_crfftop" + self.s)(self.h, z.h, x.h)
        check("vsip_crfftop")


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
