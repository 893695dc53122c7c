"""Shared-memory layout of the precision form's operand (jv_split.cu), checked
on the CPU: the step-1 and step-2 operand stores each write every (row, k)
element of the 128 x 128 16-bit A operand exactly once and stay inside it,
the step-2 stores (4-byte pairs along K) are free of bank conflicts, step 1's
16-byte stores cover 128 contiguous bytes per 8 lanes, every tcgen05.mma
operand read (two 8-column K-blocks of 16 core-matrix row groups per K = 16
chunk) ends inside A, and the four staged 1024-point rows fit the A space."""
import collections
import os
import re

SRC = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "jvsip_gb300", "csrc",
                        "jv_split.cu")).read()


def const(name):
    m = re.search(r"constexpr int %s = (\d+);" % name, SRC)
    assert m, name
    return int(m.group(1))


SPN, SPM, SPK, SPNN = const("SPN"), const("SPM"), const("SPK"), const("SPNN")
assert "SP_A_LBO = (SPM / 8) * 128 + 16;" in SRC and "SP_A_BYTES = (SPK / 8) * SP_A_LBO;" in SRC
A_LBO = (SPM // 8) * 128 + 16
A_BYTES = (SPK // 8) * A_LBO


def core_off(row, k, lbo):
    return (k >> 3) * lbo + ((row >> 3) << 7) + ((row & 7) << 4) + ((k & 7) << 1)


def all_elements():
    out = set()
    for row in range(SPM):
        for k in range(SPK):
            o = core_off(row, k, A_LBO)
            out.update((o, o + 1))
    return out


def test_step1_operand_stores():
    owner = {}
    for w in range(4):
        for l in range(32):
            base = core_off(w * 32 + l, 0, A_LBO)
            for ab in range(4):
                for part in (0, 4, 8, 12):
                    off = base + (part + ab) * A_LBO
                    assert off % 16 == 0 and off + 16 <= A_BYTES
                    for b in range(16):
                        assert off + b not in owner
                        owner[off + b] = (w, l)
    assert set(owner) == all_elements()
    # 8 lanes of a 16-byte store phase write 128 contiguous bytes
    for w in range(4):
        for l0 in range(0, 32, 8):
            offs = sorted(core_off(w * 32 + l, 0, A_LBO) for l in range(l0, l0 + 8))
            assert offs[-1] - offs[0] == 7 * 16


def test_step2_operand_stores_conflict_free():
    owner = set()
    for w in range(4):
        for c in range(32):
            mo = ((c >> 3) << 7) + ((c & 7) << 4)
            for store in range(2):
                words = collections.defaultdict(set)
                for l in range(32):
                    even = l % 2 == 0
                    k = (l if even else 96 + l - 1) if store == 0 else (32 + l if even else 64 + l - 1)
                    a = core_off(w * 32, k, A_LBO) + mo
                    assert a == core_off(w * 32 + c, k, A_LBO) and a % 4 == 0
                    for b in range(4):
                        assert a + b not in owner
                        owner.add(a + b)
                    words[(a // 4) % 32].add(a // 4)
                assert max(len(v) for v in words.values()) == 1
    assert owner == all_elements()


def test_mma_reads_and_row_stage_inside_a():
    for i in range(12):
        ka = i if i < 8 else i - 8
        start = ka * 2 * A_LBO
        # two K-blocks (lbo apart) of 16 row groups of 128 bytes
        assert start + A_LBO + (SPM // 8) * 128 <= A_BYTES
    assert 4 * SPN * 8 <= A_BYTES
