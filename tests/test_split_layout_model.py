"""Shared-memory layout of the precision form's operands (jv_split.cu), checked
on the CPU: per row group, the step-1 stores (K-major, a lane's 16-byte chunks
of 8 consecutive k) and the step-2 stores (MN-major, a lane's 16-byte chunks
of 8 consecutive m) each write every (m, k) element of the 128 x 128 16-bit A
operand exactly once and stay inside it, 8 consecutive lanes of a store write
128 contiguous bytes (no bank conflicts), every tcgen05.mma operand read ends
inside A under either reading of the descriptor's two strides, and the CTA's
shared memory (B, twiddles, four A operands) fits one SM."""
import os
import re

SRC = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "jvsip_gb300", "csrc",
                        "jv_split.cu")).read()


def const(name):
    m = re.search(r"constexpr (?:int|uint32_t) %s = ([^;]+);" % name, SRC)
    assert m, name
    return int(eval(m.group(1), {}, CONSTS))


CONSTS = {}
for _n in ("SPN", "SPM", "SPNN", "SQ_KS", "SQ_MS", "SQG", "SQW"):
    CONSTS[_n] = const(_n)
for _n in ("SP_B_LBO", "SP_B_BYTES", "SQ_A_BYTES", "SQ_TW_BYTES", "SQ_THREADS"):
    CONSTS[_n] = const(_n)
KS, MS, A_BYTES = CONSTS["SQ_KS"], CONSTS["SQ_MS"], CONSTS["SQ_A_BYTES"]


def a_off_k(m, k):
    return (m >> 3) * MS + (k >> 3) * KS + ((m & 7) << 4) + ((k & 7) << 1)


def a_off_mn(m, k):
    return (m >> 3) * MS + (k >> 3) * KS + ((k & 7) << 4) + ((m & 7) << 1)


def all_elements():
    return {o for m in range(128) for k in range(128) for o in (a_off_k(m, k), a_off_k(m, k) + 1)}


def test_layout_constants():
    assert CONSTS["SPM"] == 128 and A_BYTES == 16 * MS
    assert CONSTS["SQ_THREADS"] == CONSTS["SQG"] * CONSTS["SQW"] * 32 == 1024
    assert "a_off_k(m, ka)" in SRC and "a_off_mn(mc, lane)" in SRC
    # both layouts address the same 32 KB: (m, k) -> distinct bytes
    assert {a_off_mn(m, k) for m in range(128) for k in range(128)} == {a_off_k(m, k) for m in range(128)
                                                                         for k in range(128)}


def test_step1_operand_stores():
    owner = {}
    for r in range(4):
        for h in range(2):
            for b in range(32):
                m = 32 * r + b
                for j in range(2):
                    ka = 16 * h + 8 * j
                    for part in (0, 32, 64, 96):
                        off = a_off_k(m, part + ka)
                        assert off % 16 == 0 and off + 16 <= A_BYTES
                        for t in range(8):  # the chunk holds k = part + ka + t at off + 2t
                            assert a_off_k(m, part + ka + t) == off + 2 * t
                        for x in range(16):
                            assert off + x not in owner
                            owner[off + x] = (r, h, b)
    assert set(owner) == all_elements()
    for r in range(4):
        for b0 in range(0, 32, 8):
            offs = sorted(a_off_k(32 * r + b, 0) for b in range(b0, b0 + 8))
            assert offs[-1] - offs[0] == 7 * 16 and len(set(offs)) == 8


def test_step2_operand_stores():
    owner = {}
    for r in range(4):
        for h in range(2):
            for b in range(32):  # lane = b, the K index within each part
                for j in range(2):
                    mc = 32 * r + 16 * h + 8 * j
                    for part in (0, 32, 64, 96):
                        off = a_off_mn(mc, part + b)
                        assert off % 16 == 0 and off + 16 <= A_BYTES
                        for t in range(8):  # the chunk holds m = mc + t at off + 2t
                            assert a_off_mn(mc + t, part + b) == off + 2 * t
                        for x in range(16):
                            assert off + x not in owner
                            owner[off + x] = (r, h, b)
    assert set(owner) == all_elements()
    for b0 in range(0, 32, 8):
        offs = sorted(a_off_mn(0, b) for b in range(b0, b0 + 8))
        assert offs[-1] - offs[0] == 7 * 16 and len(set(offs)) == 8


def test_mma_reads_inside_a_either_stride_reading():
    for i in range(12):
        ka = i if i < 8 else i - 8
        start = ka * 2 * KS
        for s_m, s_k in ((MS, KS), (KS, MS)):
            last = start + 15 * s_m + 1 * s_k + 127  # 16 core matrices along m, 2 along k
            assert last < A_BYTES
    assert CONSTS["SPNN"] == 128 and CONSTS["SP_B_BYTES"] == 16 * CONSTS["SP_B_LBO"]
    for k in range(8):  # B chunks: 16 core matrices along n (128 B apart), 2 along k
        assert k * 2 * CONSTS["SP_B_LBO"] + CONSTS["SP_B_LBO"] + 16 * 128 <= CONSTS["SP_B_BYTES"]


def test_cta_shared_memory_fits():
    total = CONSTS["SP_B_BYTES"] + CONSTS["SQ_TW_BYTES"] + CONSTS["SQG"] * A_BYTES
    assert "SP_B_BYTES + SQ_TW_BYTES + SQG * SQ_A_BYTES" in SRC
    assert total + 1024 <= 227 * 1024
