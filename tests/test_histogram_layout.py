"""The counter layout of the lane-column histogram kernel (histogram_lanes_body in
cccl_gb300/csrc/radix_kernels.cuh), restated in Python: every counter address stays inside
the table the host sizes for the pass count (histogram_table_bytes), no two (pass, digit,
column) triples share a counter (a word, or a 16-bit half of one when 5-8 passes share the
words in pairs), a warp's 32 lanes hit 32 different banks in every pass, and the row bases the
fold reads cover exactly the words the counting writes."""

import pytest


def byte_perm(x, y, s):
    b = [(x >> (8 * i)) & 0xFF for i in range(4)] + [(y >> (8 * i)) & 0xFF for i in range(4)]
    return sum(b[(s >> (4 * n)) & 0xF] << (8 * n) for n in range(4))


def col(q, lane, passes):
    if passes > 4:  # two passes per 32-bit word: pass 2p in the low half, 2p + 1 in the high half
        return ((q >> 2) << 16) | (((q >> 1) & 1) * 128 + lane * 4)
    return ((q >> 1) << 16) | ((q & 1) * 128 + lane * 4)


def table_bytes(passes):
    return 65536 if passes <= 2 else 131072


def offset(q, d, lane, passes):
    # the digit sits in byte (q & 3) of the key word the kernel permutes
    word = d << (8 * (q & 3))
    return byte_perm(word, col(q, lane, passes), 0x7604 | ((q & 3) << 4))


def row_base(r, d):
    """Base of word row r (a pass, or a pair of passes when packed) for digit d, as the fold reads it."""
    return ((r >> 1) << 16) | (d << 8) | ((r & 1) * 128)


@pytest.mark.parametrize("passes", range(1, 9))
def test_lane_column_layout(passes):
    packed = passes > 4
    words = {}
    for q in range(passes):
        half = (q & 1) if packed else 0
        row = (q >> 1) if packed else q
        for d in range(256):
            offs = [offset(q, d, lane, passes) for lane in range(32)]
            assert all(o % 4 == 0 and 0 <= o < table_bytes(passes) for o in offs)
            assert offs == [row_base(row, d) + 4 * lane for lane in range(32)]
            assert sorted((o // 4) % 32 for o in offs) == list(range(32))  # conflict-free
            for lane in range(32):
                key = (offs[lane], half)
                assert key not in words, (q, d, lane, words.get(key))
                words[key] = (q, d, lane)
    # the fold's rows are exactly the counted words
    rows = (passes + 1) // 2 if packed else passes
    read = {row_base(r, d) + 4 * i for r in range(rows) for d in range(256) for i in range(32)}
    assert read == {w for w, _ in words}


def test_packed_counters_fold_before_overflow():
    """Between two folds a 16-bit half gains at most one count per warp, lane and key the
    thread loads: 32 warps x (4 loads x 2 keys x FOLD trips + head, tail and remainder keys)."""
    vec = 2  # 8-byte keys, the only ones with more than four passes
    fold = 32768 // (32 * 4 * vec) - 1
    assert 32 * (4 * vec * fold + 2 + 3 * vec) < 65536
