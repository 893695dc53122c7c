"""Autotuner of the plain c2c calls: each tuned entry (residency, radix
schedule, transforms per CTA, values per thread) lands in the versioned cache
with all its fields, plans created afterwards use it, and their results still
match the FP64 oracle within rel-L2 <= 1e-6*log2(N)."""
import ctypes as C

import numpy as np
import pytest

import jvsip_gb300 as J
import pyoracle as O

pytestmark = pytest.mark.gpu


def entry(N, cls):
    res, vpb, emax = C.c_int(), C.c_int(), C.c_int()
    rad = (C.c_int * 40)()
    n = J.lib().jvsip_fftm_autotune_plain_entry_f(N, cls, C.byref(res), C.byref(vpb), C.byref(emax), rad, 40)
    return n, res.value, vpb.value, emax.value, list(rad[:n])


def run_plan(N, count, cls, seed):
    """count transforms of N points: rows (cls 0) or columns of an N x count matrix (cls 1)."""
    x = O.fill(2 * N * count, seed, 1, np.float32)
    y = np.zeros_like(x)
    if cls == 0:
        p = J.FFTM(J.KIND_CCOP, count, N, 1.0, -1, J.VSIP_ROW)
        vx, vy = J.CBlock(x).view(0, N, count, 1, N), J.CBlock(y).view(0, N, count, 1, N)
        ref = O.CView(np.zeros(2 * N * count), 0, N, count, 1, N)
        O.Plan(O.CCOP, count, N, 1.0, O.FWD, O.ROW, np.float64).ccfftmop(
            O.CView(x.astype(np.float64), 0, N, count, 1, N), ref)
    else:
        p = J.FFTM(J.KIND_CCOP, N, count, 1.0, -1, J.VSIP_COL)
        vx, vy = J.CBlock(x).view(0, count, N, 1, count), J.CBlock(y).view(0, count, N, 1, count)
        ref = O.CView(np.zeros(2 * N * count), 0, count, N, 1, count)
        O.Plan(O.CCOP, N, count, 1.0, O.FWD, O.COL, np.float64).ccfftmop(
            O.CView(x.astype(np.float64), 0, count, N, 1, count), ref)
    p.ccfftmop(vx, vy)
    err = np.linalg.norm(y.astype(np.float64) - ref.buf) / np.linalg.norm(ref.buf)
    return p, err


ROOT = __import__("os").path.dirname(__import__("os").path.dirname(__import__("os").path.abspath(__file__)))


def child(code, cache):
    """Run `code` in a fresh process whose tuner cache is `cache` (tuned
    entries are process-wide: they would change the kernels of later tests)."""
    import os
    import subprocess
    import sys
    env = dict(os.environ, JVSIP_GPU_TUNE_CACHE=str(cache))
    pre = "import sys; sys.path.insert(0, 'tests'); sys.path.insert(0, 'oracle'); import test_gpu_tune as T; "
    return subprocess.check_output([sys.executable, "-c", pre + code], env=env, cwd=ROOT, text=True)


@pytest.mark.parametrize("N,cls", [(1000, 0), (1536, 0), (768, 0), (4096, 0), (1000, 1), (2048, 1), (96, 0)])
def test_plain_tuner_entry_is_cached_used_and_correct(N, cls, tmp_path):
    cache = tmp_path / "tune.txt"
    out = child("import ctypes as C; L = T.J.lib(); "
                "assert L.jvsip_fftm_autotune_plain_f(1, (C.c_ulong * 1)(%d), %d) == 0, T.J.last_error(); "
                "p, err = T.run_plan(%d, 48, %d, %d); print(T.entry(%d, %d), p.passes(), err)"
                % (N, cls, N, cls, N + cls, N, cls), cache)
    lines = [ln.split() for ln in cache.read_text().splitlines() if ln.startswith("P ")]
    assert len(lines) == 1
    f = lines[0]
    n_, prec, c_, res, vpb, emax, npass = (int(v) for v in f[2:9])
    radices = [int(v) for v in f[9:]]
    assert (n_, prec, c_) == (N, 0, cls) and res in (0, 1) and emax in (0, 8, 16) and vpb >= 0
    assert npass == len(radices) and int(np.prod(radices)) == N
    ent, passes, err = out.strip().split(") ")[0] + ")", "[" + out.split("[", 2)[2].split("]")[0] + "]", out.split()[-1]
    assert ent == str((npass, res, vpb, emax, radices))
    assert passes == str(radices)       # the plan created after tuning uses the tuned schedule
    assert float(err) <= 1e-6 * np.log2(N), f"rel-L2 {err}"


def test_cache_line_with_another_schedule_is_applied_by_a_new_process(tmp_path):
    # an entry of the shared-memory kernel with a non-default schedule
    # (640 = 10 x 8 x 8 rather than the default 16 x 10 x 4), written as a
    # cache line, is what plan creation applies in a fresh process, and that
    # plan still matches the oracle
    cache = tmp_path / "tune.txt"
    child("import ctypes as C; L = T.J.lib(); "
          "assert L.jvsip_fftm_autotune_plain_f(1, (C.c_ulong * 1)(640), 0) == 0", cache)
    f = [ln for ln in cache.read_text().split("\n") if ln.startswith("P ")][0].split()
    # P gpu N prec cls res vpb emax npasses radices...
    f[5] = "1"
    f[8:] = ["3", "10", "8", "8"]
    cache.write_text(" ".join(f) + "\n")
    out = child("p, err = T.run_plan(640, 16, 0, 7); print(p.passes(), err)", cache)
    passes, err = out.strip().rsplit(" ", 1)
    assert passes == "[10, 8, 8]"
    assert float(err) <= 1e-6 * np.log2(640)
