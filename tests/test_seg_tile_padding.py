"""The padding arithmetic of the segmented device-class pass (seg_device_persistent_body in
cccl_gb300/csrc/segmented_kernels.cuh), restated on the CPU for every tile shape the pass can
have and every fill of a segment's last tile.

Warp w of the main threads holds tile slots [w * WS, (w + 1) * WS), WS = 32 x items. Warps whose
slots all lie past the tile's `valid` keys (padding-only warps) skip the digit count; their
padding keys still rank, after every counted key, from the running offsets the look-back
threads leave in the warps' rows. The look-back threads discount only the counted padding
(`counted - valid`, counted = the live warps' slots) when they test for a single-digit tile.
The checks: the counted slots cover the real keys and are never clipped by the tile, the
live warps are exactly those below `valid`, and the positions the padding-only warps rank into
stay inside the staged tile."""

import pytest


def live_warps(valid, ws):
    return -(-valid // ws)


@pytest.mark.parametrize("main_threads", [640, 768])
@pytest.mark.parametrize("items", range(1, 17))
def test_padding_only_warps_stay_inside_the_tile(main_threads, items):
    ws = 32 * items
    warps = main_threads // 32
    tile = warps * ws
    for valid in range(1, tile + 1):
        live = live_warps(valid, ws)
        counted = min(tile, live * ws)  # the kernel's formula
        assert counted == live * ws  # never clipped: live <= warps
        assert valid <= counted < valid + ws  # the live warps hold every real key
        # a warp is live iff its first slot is below valid
        assert all((w * ws < valid) == (w < live) for w in range(warps))
        # digit dmask holds the real keys of that digit, then the counted padding; the
        # padding-only warps count nothing, so each ranks its keys from `counted` on
        if live < warps:
            assert counted + ws <= tile  # their positions [counted, counted + ws)
