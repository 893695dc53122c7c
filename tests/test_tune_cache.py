"""The autotuner's versioned cache file, read on the host: a plain-call line
(P gpu N prec cls res vpb emax npasses radices...) and a batch line
(B gpu N prec vf per) are parsed into the entries the library applies; lines of
another GPU, malformed lines and other stride classes are ignored. Runs without
a GPU (the cache is keyed by the name "gpu" there) in a fresh process, since a
process reads the cache once."""
import os
import subprocess
import sys

import pytest

import jvsip_gb300 as J

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROBE = r'''
import ctypes as C, jvsip_gb300 as J
L = J.lib()
def entry(N, cls):
    r, v, e = C.c_int(), C.c_int(), C.c_int()
    rad = (C.c_int * 40)()
    n = L.jvsip_fftm_autotune_plain_entry_f(N, cls, C.byref(r), C.byref(v), C.byref(e), rad, 40)
    return (n, r.value, v.value, e.value, list(rad[:n]))
print(entry(640, 0)); print(entry(640, 1)); print(entry(1000, 0)); print(entry(96, 0))
print(L.jvsip_fftm_autotune_entries())
'''


def test_cache_lines_are_parsed(tmp_path):
    if J.gpu_available():
        pytest.skip("the host-side cache key is used only without a GPU")
    cache = tmp_path / "tune.txt"
    cache.write_text("P gpu 640 0 0 1 4 16 3 10 8 8\n"
                     "P other_gpu 1000 0 0 1 2 8 3 10 10 10\n"
                     "P gpu 96 0 0 1 garbage\n"
                     "B gpu 4096 0 1 4\n"
                     "P gpu 1000 0 1 0 0 0 3 10 10 10\n")
    env = dict(os.environ, JVSIP_GPU_TUNE_CACHE=str(cache))
    out = subprocess.check_output([sys.executable, "-c", PROBE], env=env, cwd=ROOT, text=True).split("\n")
    assert out[0] == "(3, 1, 4, 16, [10, 8, 8])"       # P line of this GPU, class 0
    assert out[1] == "(0, 0, 0, 0, [])"                 # no class-1 entry for 640
    assert out[2] == "(0, 0, 0, 0, [])"                 # 1000 class 0 only for another GPU
    assert out[3] == "(0, 0, 0, 0, [])"                 # malformed line ignored
    assert int(out[4]) == 3                             # 640/0, 1000/1 and the batch entry
