"""Index model of the register-resident kernel (jvsip_gb300/csrc/jv_fast.cuh),
checked on the CPU for every instance the launchers create (read from
jv_fast.cu and jv_fast_real.cu): the schedule is the plan's (fast_radices,
whose per-pass twiddle tables the kernel indexes), every pass reads and writes
each of the N points exactly once, shared-memory indices stay inside the
CTA's allocation, the allocation fits an SM, the R2C split writes bins
0..N exactly once and the C2R merge reads only bins 0..N, and the
shared-memory exchanges of power-of-two transforms are free of bank conflicts
(the padding and pitch rules of fast_pad_shift / fast_pitch, restated here)."""
import os
import re

import numpy as np
import pytest

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "jvsip_gb300", "csrc")
SMEM_MAX = 227 * 1024


def sources():
    return {f: open(os.path.join(CSRC, f)).read() for f in ("jv_fast.cu", "jv_fast_real.cu")}


def fast_radices():
    src = sources()["jv_fast.cu"]
    body = src[src.index("std::vector<int> fast_radices(long N)"):]
    body = body[:body.index("default:")]
    return {int(n): [int(r) for r in rs.split(",")] for n, rs in re.findall(r"case (\d+): return \{([\d, ]+)\};", body)}


def instances():
    """(file, N, T, RPC, radices, cols, sp, rm) of every launch_fast_n<...> case."""
    out = []
    pat = re.compile(r"case (\d+): return launch_fast_n<(\d+), (\d+), (\d+), RList<([\d, ]+)>, ([^>]*)>\(j, st\);")
    for f, src in sources().items():
        for m in pat.finditer(src):
            n_case, N, T, RPC, rl, rest = m.groups()
            assert int(n_case) == int(N)
            args = [a.strip() for a in rest.split(",")]
            cols = args[1] == "true"
            sp = len(args) > 3 and args[3] == "true"
            rms = [0]
            if len(args) > 4:
                rms = [1, 2] if args[4] == "RM" else [int(args[4])]
            for rm in rms:
                out.append((f, int(N), int(T), int(RPC), [int(r) for r in rl.split(",")], cols, sp, rm))
    return out


def pad_shift(N):
    return 5 if N in (1000, 768) else 4


def padx(i, N):
    return i + (i >> pad_shift(N))


def pitch(N, RPC, cols):
    base = N + (N >> pad_shift(N))
    if not cols:
        return base
    if RPC > 8:
        return base + 1
    return base + (16 // RPC - base % 16 + 16) % 16


def ids(inst):
    f, N, T, RPC, rad, cols, sp, rm = inst
    return f"{f[:-3]}-{N}-T{T}-R{RPC}-{'cols' if cols else 'rows'}{'-sp' if sp else ''}{'-rm%d' % rm if rm else ''}"


INST = instances()


def test_instances_found():
    assert len(INST) >= 40
    assert {N for _, N, *_ in INST} >= {64, 128, 256, 512, 768, 1000, 1024, 2048, 4096, 8192}


@pytest.mark.parametrize("inst", INST, ids=ids)
def test_schedule_and_passes(inst):
    f, N, T, RPC, rad, cols, sp, rm = inst
    # the kernel's schedule is the plan's: its twiddle tables follow fast_radices
    assert fast_radices()[N] == rad
    assert int(np.prod(rad)) == N and N % T == 0 and T * RPC <= 1024
    E = N // T
    assert all(E % R == 0 for R in rad)
    t = np.arange(T)
    # first pass: global reads of element t + T*b + r*N/R1
    R1 = rad[0]
    n = (t[:, None, None] + T * np.arange(E // R1)[None, :, None] + (N // R1) * np.arange(R1)[None, None, :]).ravel()
    assert np.array_equal(np.sort(n), np.arange(N))
    NP = pitch(N, RPC, cols)
    assert RPC * NP * 8 <= SMEM_MAX
    Ns = 1
    for p, R in enumerate(rad):
        B = E // R
        j = (t[:, None] + T * np.arange(B)[None, :]).ravel()
        assert j.max() < N // R
        if p > 0:
            # load: t + T*b + r*N/R
            li = (j[:, None] + (N // R) * np.arange(R)[None, :]).ravel()
            assert np.array_equal(np.sort(li), np.arange(N))
        m = j % Ns
        si = (((j - m) * R + m)[:, None] + Ns * np.arange(R)[None, :]).ravel()
        assert np.array_equal(np.sort(si), np.arange(N))
        # padded indices inside the transform's row, rows inside the allocation
        assert padx(si.max(), N) < NP and padx(N - 1, N) < NP
        Ns *= R
    assert Ns == N


@pytest.mark.parametrize("inst", [i for i in INST if i[7] != 0], ids=ids)
def test_real_rows(inst):
    f, N, T, RPC, rad, cols, sp, rm = inst
    assert not cols and not sp
    t = np.arange(T)
    if rm == 1:
        # R2C split: the thread of pair k (k = t + T*i <= N/2) writes X_k and X_{N-k} (X_N for k = 0)
        npair = N // 2 + 1
        k = (t[:, None] + T * np.arange((npair + T - 1) // T)[None, :]).ravel()
        k = k[k < npair]
        nk = np.where(k == 0, N, N - k)
        written = np.concatenate([k, nk[nk != k]])
        assert np.array_equal(np.sort(written), np.arange(N + 1))
        # reads Z_k and Z_{N-k} (Z_N = Z_0) inside the transform's row
        assert max(k.max(), (N - k[k > 0]).max()) < N
    else:
        # C2R merge: element n reads X_n and X_{N-n} (X_N at n = 0), bins 0..N
        n = np.arange(N)
        assert (N - n).max() == N and (N - n).min() == 1


def wavefronts(idx):
    """64-bit accesses of one half-warp: the largest number of distinct
    elements that share a bank."""
    banks = {}
    for e in set(idx):
        for w in (2 * e, 2 * e + 1):
            banks.setdefault(w % 32, set()).add(e)
    return max(len(v) for v in banks.values())


def mean_wavefronts(N, T, RPC, rad, cols):
    NP = pitch(N, RPC, cols)
    E = N // T
    nthr = T * RPC
    tot = cnt = 0
    Ns = 1
    for p, R in enumerate(rad):
        for phase in ("load", "store"):
            if (p == 0 and phase == "load") or (p == len(rad) - 1 and phase == "store"):
                continue
            for b in range(E // R):
                for r in range(R):
                    for h in range(0, nthr, 16):
                        idx = []
                        for tid in range(h, min(h + 16, nthr)):
                            tt, rl = (tid // RPC, tid % RPC) if cols else (tid % T, tid // T)
                            if phase == "load":
                                i = tt + T * b + r * (N // R)
                            else:
                                j = tt + T * b
                                m = j % Ns
                                i = (j - m) * R + m + r * Ns
                            idx.append(rl * NP + padx(i, N))
                        tot += wavefronts(idx)
                        cnt += 1
        Ns *= R
    return tot / cnt


@pytest.mark.parametrize("inst", [i for i in INST if not i[6] and i[7] == 0 and i[1] & (i[1] - 1) == 0 and i[1] <= 4096],
                         ids=ids)
def test_power_of_two_exchanges_conflict_free(inst):
    f, N, T, RPC, rad, cols, sp, rm = inst
    assert mean_wavefronts(N, T, RPC, rad, cols) == 1.0


@pytest.mark.parametrize("N,T,RPC,rad,cols,bound", [(768, 32, 4, [12, 8, 8], False, 1.5),
                                                    (1000, 100, 4, [10, 10, 10], False, 1.7),
                                                    (1000, 100, 4, [10, 10, 10], True, 1.25)])
def test_mixed_radix_exchanges(N, T, RPC, rad, cols, bound):
    assert mean_wavefronts(N, T, RPC, rad, cols) <= bound
