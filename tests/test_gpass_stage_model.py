"""Index model of the multi-pass global path's first pass with staged stores
(k_gpass_r1 in jv_kernels.cuh), run on the CPU: every CTA trip writes its
butterflies' R outputs into shared-memory slots t*P + r (P = R | 1) and reads
them back as element e -> slot (e // R)*P + e % R for output j*R + r of the
slot's transform; over all trips every output of every transform is written
exactly once, every slot index stays inside the 256*P staging, a half-warp's
64-bit staging stores hit 16 distinct bank pairs, and the launcher's size
check keeps the staging plus the slot indices inside 48 KB.  Also the odd-prime
codelet's root constants against cos / sin of 2 pi k / R."""
import math
import pathlib
import re

import numpy as np
import pytest

SRC = pathlib.Path(__file__).resolve().parents[1] / "jvsip_gb300" / "csrc" / "jv_kernels.cuh"
CODELETS = [2, 3, 4, 5, 6, 7, 8, 9, 10, 12, 14, 15, 16, 11, 13, 17, 19, 23]


def pitch(R):
    return R | 1


def staged_launch(R, esz):
    """The launcher's condition for the staged first pass."""
    return 256 * pitch(R) * 2 * esz + 256 * 12 <= 48 * 1024


@pytest.mark.parametrize("R", CODELETS)
@pytest.mark.parametrize("N_over_R,nvec,grid", [(704, 3, 4), (11, 40, 3), (1, 300, 2), (257, 2, 5), (4, 7, 1)])
def test_first_pass_staging_covers_every_output_once(R, N_over_R, nvec, grid):
    N, NR = R * N_over_R, N_over_R
    total = nvec * NR
    P = pitch(R)
    seen = np.zeros((nvec, N), np.int32)
    for b in range(grid):
        i0 = b * 256
        while i0 < total:
            slots = {}
            for t in range(256):
                i = i0 + t
                if i < total:
                    v, j = divmod(i, NR)
                    for r in range(R):
                        assert 0 <= t * P + r < 256 * P
                    slots[t] = (v, j)
            cnt = min(total - i0, 256) * R
            for e in range(cnt):
                q, r = divmod(e, R)
                assert q in slots and q * P + r < 256 * P
                v, j = slots[q]
                seen[v, j * R + r] += 1
            i0 += grid * 256
    assert (seen == 1).all()


@pytest.mark.parametrize("R", CODELETS)
def test_staging_stores_hit_distinct_banks(R):
    P = pitch(R)
    for r in range(R):
        banks = [((t * P + r) * 2) % 32 for t in range(16)]  # 64-bit: word pair (b, b+1)
        assert len(set(banks)) == 16


def test_launch_condition_fits_default_shared_memory():
    for R in CODELETS:
        for esz in (4, 8):
            if staged_launch(R, esz):
                assert 256 * pitch(R) * 2 * esz + 256 * (8 + 4) <= 49152
    # single precision stages every radix up to 19; radix 23 (47104 + 3072 bytes) does not
    assert all(staged_launch(R, 4) for R in CODELETS if R <= 19)
    assert not staged_launch(23, 4)


def test_prime_root_constants():
    text = SRC.read_text()
    for R in (11, 13, 17, 19, 23):
        for name, fn in (("cos", math.cos), ("sin", math.sin)):
            m = re.search(r"prime_%s<%d>\(int i\) \{(.*?)\}" % (name, R), text, re.S)
            assert m, (name, R)
            vals = [float(x) for x in re.findall(r"-?\d+\.\d+(?:e-?\d+)?", m.group(1))]
            H = (R - 1) // 2
            assert len(vals) == H
            for k, val in enumerate(vals, start=1):
                assert abs(val - fn(2 * math.pi * k / R)) <= 2e-16
