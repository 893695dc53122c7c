"""Batching form: many independent c2c fftm calls of uneven 2^a 3^b 5^c
lengths, row counts, directions and majors in one launch, direct and captured
(CUDA-graph replay), against the per-plan calls and the FP64 oracle; the
autotuner's cache; rejection of unsupported inputs."""
import ctypes as C
import os

import numpy as np
import pytest

import jvsip_gb300 as J
import pyoracle as O
from jvsip_gb300 import synth

pytestmark = pytest.mark.gpu


def make_batch(seq, seed=3):
    total = sum(N * r for N, r, _, _ in seq)
    x = O.fill(2 * total, seed, 1, np.float32)
    y = np.zeros_like(x)
    bx, by = J.CBlock(x), J.CBlock(y)
    bx.admit(True)
    by.admit(False)
    plans, vin, vout, offs = [], [], [], []
    off = 0
    for N, r, d, major in seq:
        scale = 1.0 if d == -1 else 1.0 / N
        if major == 0:
            plans.append(J.FFTM(J.KIND_CCOP, r, N, scale, d, J.VSIP_ROW))
            vin.append(bx.view(off, N, r, 1, N))
            vout.append(by.view(off, N, r, 1, N))
        else:
            plans.append(J.FFTM(J.KIND_CCOP, N, r, scale, d, J.VSIP_COL))
            vin.append(bx.view(off, r, N, 1, r))
            vout.append(by.view(off, r, N, 1, r))
        offs.append(off)
        off += N * r
    n = len(seq)
    arrs = ((C.c_void_p * n)(*[p.h for p in plans]), (C.c_void_p * n)(*[v.h for v in vin]),
            (C.c_void_p * n)(*[v.h for v in vout]))
    return x, y, bx, by, plans, vin, vout, offs, arrs


def oracle_check(seq, x, y, offs):
    worst = 0.0
    for (N, r, d, major), off in zip(seq, offs):
        scale = 1.0 if d == -1 else 1.0 / N
        xs = O.CView(x[2 * off:2 * (off + N * r)].astype(np.float64), 0,
                     N if major == 0 else 1, r if major == 0 else N, 1 if major == 0 else r, N if major == 0 else r)
        # VSIP_COL: an N x r matrix (col_stride r, row_stride 1) transformed along its columns
        if major == 1:
            xs = O.CView(x[2 * off:2 * (off + N * r)].astype(np.float64), 0, r, N, 1, r)
            ys = O.CView(np.zeros(2 * N * r), 0, r, N, 1, r)
            O.Plan(O.CCOP, N, r, scale, d, O.COL, np.float64).ccfftmop(xs, ys)
        else:
            xs = O.CView(x[2 * off:2 * (off + N * r)].astype(np.float64), 0, N, r, 1, N)
            ys = O.CView(np.zeros(2 * N * r), 0, N, r, 1, N)
            O.Plan(O.CCOP, r, N, scale, d, O.ROW, np.float64).ccfftmop(xs, ys)
        got = y[2 * off:2 * (off + N * r)].astype(np.float64)
        err = np.linalg.norm(got - ys.buf) / np.linalg.norm(ys.buf)
        assert err <= 1e-6 * np.log2(N), (N, r, d, major, err)
        worst = max(worst, err)
    return worst


SEQ = synth.batch_sequence(40, seed=11, max_bytes=64e6)


def test_batch_matches_oracle_direct_and_captured():
    L = J.lib()
    x, y, bx, by, plans, vin, vout, offs, (P, VI, VO) = make_batch(SEQ)
    assert L.jvsip_fftm_batch_f(len(SEQ), P, VI, VO) == 0, J.last_error()
    by.sync()
    oracle_check(SEQ, x, y, offs)
    first = y.copy()
    # captured: build once, replay twice
    y[:] = 0
    by.admit(True)   # re-upload zeros so the replay is what fills the output
    bp = L.jvsip_fftm_batch_create_f(len(SEQ), P, VI, VO)
    assert bp, J.last_error()
    for _ in range(2):
        assert L.jvsip_fftm_batch_run_f(bp) == 0
    by.sync()
    assert np.array_equal(y, first)
    assert L.jvsip_fftm_batch_destroy_f(bp) == 0


def test_batch_equals_per_plan_calls():
    L = J.lib()
    x, y, bx, by, plans, vin, vout, offs, (P, VI, VO) = make_batch(SEQ, seed=4)
    for i in range(len(SEQ)):
        L.vsip_ccfftmop_f(P[i], VI[i], VO[i])
    by.sync()
    loop = y.copy()
    assert L.jvsip_fftm_batch_f(len(SEQ), P, VI, VO) == 0
    by.sync()
    # same kernels' arithmetic except the row kernel for power-of-two rows: compare to tolerance
    assert np.linalg.norm(y - loop) / np.linalg.norm(loop) < 1e-6


def test_loop_from_c_equals_per_plan_calls():
    L = J.lib()
    x, y, bx, by, plans, vin, vout, offs, (P, VI, VO) = make_batch(SEQ[:12], seed=5)
    assert L.jvsip_fftm_loop_f(12, P, VI, VO) == 0, J.last_error()
    by.sync()
    oracle_check(SEQ[:12], x, y, offs)
    assert L.jvsip_fftm_loop_f(0, None, None, None) == 0


def test_batch_rejects_unsupported():
    L = J.lib()
    x = np.zeros(2 * 64 * 11, np.float32)
    b = J.CBlock(x)
    v = b.view(0, 11 * 64, 1, 1, 11 * 64)
    p = J.FFTM(J.KIND_CCIP, 1, 11 * 64, 1.0, -1, J.VSIP_ROW)   # prime factor 11
    P, V = (C.c_void_p * 1)(p.h), (C.c_void_p * 1)(v.h)
    b.admit(True)
    assert L.jvsip_fftm_batch_f(1, P, V, V) != 0
    L.jvsip_gpu_clear_error()
    q = J.FFTM(J.KIND_CCIP, 1, 64, 1.0, -1, J.VSIP_ROW)
    w = J.CBlock(np.zeros(128, np.float32))     # not admitted
    vw = w.view(0, 64, 1, 1, 64)
    assert L.jvsip_fftm_batch_f(1, (C.c_void_p * 1)(q.h), (C.c_void_p * 1)(vw.h), (C.c_void_p * 1)(vw.h)) != 0
    code, msg = J.last_error()
    assert "admitted" in msg
    L.jvsip_gpu_clear_error()


def test_autotune_cache(tmp_path, monkeypatch):
    L = J.lib()
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("JVSIP_GPU_TUNE_CACHE", str(cache))
    lens = (C.c_ulong * 3)(64, 1000, 4096)
    assert L.jvsip_fftm_autotune_f(3, lens, 0) == 0
    assert L.jvsip_fftm_autotune_entries() >= 3
    text = cache.read_text().split("\n")
    assert len([t for t in text if t.strip()]) >= 3
    # tuned tiles are still correct
    seq = [(1000, 37, -1, 0), (64, 200, 1, 1), (4096, 3, 1, 0)]
    x, y, bx, by, plans, vin, vout, offs, (P, VI, VO) = make_batch(seq, seed=8)
    assert L.jvsip_fftm_batch_f(len(seq), P, VI, VO) == 0
    by.sync()
    oracle_check(seq, x, y, offs)


def test_batch_long_columns_through_the_plain_two_steps():
    """Columns of 8192+ points (adjacent, more than one) run through the plain
    calls' two steps on streams of their own beside the tile launches (one
    plan's calls on one stream); a single long column keeps the cluster kernel,
    shorter columns the tiles.  Direct and captured (replayed twice), in place,
    against the FP64 oracle."""
    L = J.lib()
    seq = [(16384, 40, -1, 1), (10000, 7, 1, 1), (8192, 100, 1, 1), (12288, 1, -1, 1), (1000, 30, -1, 0),
           (3125, 30, -1, 1), (64, 50, 1, 1), (4096, 20, 1, 1)]
    x, y, bx, by, plans, vin, vout, offs, (P, VI, VO) = make_batch(seq, seed=12)
    assert L.jvsip_fftm_batch_f(len(seq), P, VI, VO) == 0, J.last_error()
    by.sync()
    oracle_check(seq, x, y, offs)
    direct = y.copy()
    y[:] = 0
    by.admit(True)   # re-upload zeros so the replay is what fills the output
    bp = L.jvsip_fftm_batch_create_f(len(seq), P, VI, VO)
    assert bp, J.last_error()
    for _ in range(2):
        assert L.jvsip_fftm_batch_run_f(bp) == 0
    by.sync()
    assert np.array_equal(y, direct)
    assert L.jvsip_fftm_batch_destroy_f(bp) == 0
    # in place: x and y the same view
    x2, _, bx2, _, plans2, vin2, _, offs2, (P2, VI2, _) = make_batch(seq, seed=13)
    x0 = x2.copy()
    assert L.jvsip_fftm_batch_f(len(seq), P2, VI2, VI2) == 0, J.last_error()
    bx2.sync()
    oracle_check(seq, x0, x2, offs2)
    # only long columns on the plain path: two plans on the plain-path streams, direct and captured
    seq3 = [(16384, 12, -1, 1), (8192, 9, 1, 1)]
    x3, y3, bx3, by3, plans3, vin3, vout3, offs3, (P3, VI3, VO3) = make_batch(seq3, seed=14)
    assert L.jvsip_fftm_batch_f(len(seq3), P3, VI3, VO3) == 0, J.last_error()
    by3.sync()
    oracle_check(seq3, x3, y3, offs3)
    bp3 = L.jvsip_fftm_batch_create_f(len(seq3), P3, VI3, VO3)
    assert bp3, J.last_error()
    y3[:] = 0
    by3.admit(True)
    assert L.jvsip_fftm_batch_run_f(bp3) == 0
    by3.sync()
    oracle_check(seq3, x3, y3, offs3)
    assert L.jvsip_fftm_batch_destroy_f(bp3) == 0
