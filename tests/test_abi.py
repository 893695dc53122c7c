"""CPU-side checks of the C ABI: the library builds, loads, exports every
symbol the public header declares, its VSIPL object layouts match the
reference's byte for byte, and without a GPU plan creation fails cleanly."""
import ctypes as C
import os
import re
import subprocess

import pytest

import jvsip_gb300 as J

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "vsip_fftm_gb300.h")


def header_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set(re.findall(r"\b((?:vsip|jvsip)_\w+)\s*\(", text))
    return sorted(names)


def test_header_declares_what_the_package_lists():
    assert set(header_functions()) == set(J.EXPORTS)


def test_library_exports_every_declared_symbol():
    L = J.lib()
    missing = [s for s in header_functions() if not hasattr(L, s)]
    assert missing == []


def test_header_compiles_as_c89_and_c99(tmp_path):
    src = tmp_path / "h.c"
    src.write_text('#include "vsip_fftm_gb300.h"\nint main(void){ return 0; }\n')
    for std in ("-std=c89", "-std=c99"):
        subprocess.check_call(["gcc", std, "-pedantic", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                               "-c", str(src), "-o", str(tmp_path / "h.o")])


LAYOUT_PROBE = r'''
#include <stdio.h>
#include <stddef.h>
#include "jvsip_gb300/csrc/vsip_layout.h"
#define O(s, f) (unsigned long)offsetof(struct s, f)
int main(void) {
  printf("%lu %lu %lu %lu %lu %lu %lu %lu\n", (unsigned long)sizeof(struct vsip_cblockattributes_f),
         O(vsip_cblockattributes_f, cstride), O(vsip_cblockattributes_f, a_scalar), O(vsip_cblockattributes_f, update),
         (unsigned long)sizeof(struct vsip_cblockattributes_d), O(vsip_cblockattributes_d, update),
         (unsigned long)sizeof(struct vsip_blockattributes_f), O(vsip_blockattributes_f, update));
  printf("%lu %lu %lu %lu\n", (unsigned long)sizeof(struct vsip_cmviewattributes_f),
         O(vsip_cmviewattributes_f, col_length), (unsigned long)sizeof(struct vsip_mviewattributes_d),
         O(vsip_mviewattributes_d, markings));
  printf("%lu %lu %lu %lu\n", (unsigned long)sizeof(struct vsip_fftmattributes_f),
         O(vsip_fftmattributes_f, scale), O(vsip_fftmattributes_f, MN), O(vsip_fftmattributes_f, ext_fftm_obj));
  printf("%lu %lu %lu %lu %lu %lu\n", (unsigned long)sizeof(struct vsip_vviewattributes_f),
         O(vsip_vviewattributes_f, length), O(vsip_vviewattributes_f, markings),
         (unsigned long)sizeof(struct vsip_cvviewattributes_d), O(vsip_cvviewattributes_d, stride),
         O(vsip_cvviewattributes_d, markings));
  printf("%lu %lu %lu %lu %lu %lu\n", (unsigned long)sizeof(struct vsip_fftattributes_f),
         O(vsip_fftattributes_f, scale), O(vsip_fftattributes_f, N), O(vsip_fftattributes_f, ext_fft_obj),
         (unsigned long)sizeof(struct vsip_fftattributes_d), O(vsip_fftattributes_d, ext_fft_obj));
  printf("%lu %lu\n", (unsigned long)sizeof(vsip_fft_attr_f), (unsigned long)sizeof(vsip_fft_attr_d));
  return 0; }
'''
# sizes and offsets of the reference's default build on LP64 hosts
# (c_VSIP_src/vsip_cblockattributes_f.h:42-67, vsip_blockattributes_f.h:40-51,
#  vsip_cmviewattributes_f.h:47-55, vsip_fftmattributes_f.h:8-38,
#  vsip_vviewattributes_f.h:46-52, vsip_cvviewattributes_d.h, vsip_fftattributes_f.h:8-31,
#  vsip.h:275-276)
LAYOUT_REF = ["88 24 52 84 128 120 56 52", "56 40 56 48", "256 160 184 248", "40 24 32 40 16 32",
              "176 112 120 168 176 168", "32 40"]


def test_object_layouts_match_the_reference(tmp_path):
    src = tmp_path / "layout.c"
    src.write_text(LAYOUT_PROBE)
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-std=c99", "-I", ROOT, str(src), "-o", str(exe)])
    out = subprocess.check_output([str(exe)], text=True).split("\n")[:6]
    assert out == LAYOUT_REF


def test_no_gpu_create_returns_null_with_error():
    if J.gpu_available():
        pytest.skip("a GPU is present")
    L = J.lib()
    L.jvsip_gpu_clear_error()
    assert L.vsip_ccfftmop_create_f(4, 16, 1.0, -1, 0, 0, 0) is None
    code, msg = J.last_error()
    assert code == 1 and "device" in msg
    assert L.vsip_fftm_destroy_f(None) == 0
    assert L.vsip_ccfftop_create_f(1024, 1.0, -1, 0, 0) is None
    assert L.vsip_rcfftop_create_d(1024, 1.0, 0, 0) is None
    assert L.vsip_fft_destroy_f(None) == 0
    assert L.vsip_fft_destroy_d(None) == 0


def test_plan_of_a_long_prime_length_is_refused_before_any_device_work():
    # 1024 rows of the prime length 1048573 are direct sums of about 1.1e12
    # complex multiply-adds per call; plan creation refuses them (on any host)
    L = J.lib()
    L.jvsip_gpu_clear_error()
    assert L.vsip_ccfftmop_create_f(1024, 1048573, 1.0, -1, 0, 0, 0) is None
    code, msg = J.last_error()
    assert "refused" in msg and "multiply-adds" in msg, msg
    L.jvsip_gpu_clear_error()
    assert L.vsip_ccfftop_create_d(1048573, 1.0, -1, 0, 0) is None
    code, msg = J.last_error()
    assert "refused" in msg, msg
    L.jvsip_gpu_clear_error()


def test_block_lifecycle_without_gpu():
    import numpy as np
    L = J.lib()
    a = np.zeros(32, np.float32)
    b = L.vsip_cblockbind_f(a.ctypes.data, None, 16, 0)
    assert b
    v = L.vsip_cmbind_f(b, 0, 4, 4, 1, 4)
    assert v
    assert L.vsip_cmdestroy_f(v) == b
    w = L.vsip_cvbind_f(b, 2, -1, 3)
    assert w
    assert L.vsip_cvdestroy_f(w) == b
    L.vsip_cblockdestroy_f(b)
