"""The counter layout of the lane-column histogram kernel (histogram_lanes_body in
cccl_gb300/csrc/radix_kernels.cuh), restated in Python: every counter address stays inside
the table the host sizes for the pass count (histogram_table_bytes), no two (pass, digit,
column) triples share a word, a warp's 32 lanes hit 32 different banks in passes 0-3, and
the row bases the reduction reads cover exactly the words the counting writes."""

import pytest


def byte_perm(x, y, s):
    b = [(x >> (8 * i)) & 0xFF for i in range(4)] + [(y >> (8 * i)) & 0xFF for i in range(4)]
    return sum(b[(s >> (4 * n)) & 0xF] << (8 * n) for n in range(4))


def col(q, lane):
    if q < 4:
        return ((q >> 1) << 16) | ((q & 1) * 128 + lane * 4)
    return (2 << 16) | ((q & 3) * 64 + (lane & 15) * 4)


def table_bytes(passes):
    return 65536 if passes <= 2 else 131072 if passes <= 4 else 196608


def offset(q, d, lane):
    # the digit sits in byte (q & 3) of the key word the kernel permutes
    word = d << (8 * (q & 3))
    return byte_perm(word, col(q, lane), 0x7604 | ((q & 3) << 4))


def row_base(q, d):
    if q < 4:
        return ((q >> 1) << 16) | (d << 8) | ((q & 1) * 128)
    return (2 << 16) | (d << 8) | ((q & 3) * 64)


@pytest.mark.parametrize("passes", range(1, 9))
def test_lane_column_layout(passes):
    words = {}
    for q in range(passes):
        width = 32 if q < 4 else 16
        for d in range(256):
            offs = [offset(q, d, lane) for lane in range(32)]
            assert all(o % 4 == 0 and 0 <= o < table_bytes(passes) for o in offs)
            assert offs == [row_base(q, d) + 4 * (lane % width) for lane in range(32)]
            if q < 4:
                assert sorted((o // 4) % 32 for o in offs) == list(range(32))  # conflict-free
            for lane in range(width):
                key = offs[lane]
                assert key not in words, (q, d, lane, words.get(key))
                words[key] = (q, d, lane)
    # the reduction's rows are exactly the counted words
    rows = {row_base(q, d) + 4 * i for q in range(passes) for d in range(256) for i in range(32 if q < 4 else 16)}
    assert rows == set(words)
