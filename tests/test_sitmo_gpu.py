"""The device sitmo block function against the reference engine's known answers."""
import numpy as np
import pytest

import pyoracle as O

pytestmark = pytest.mark.gpu


def test_device_blocks_match_reference_kat(golden, ctx):
    for line in golden("sitmo_kat.txt").strip().splitlines():
        head, vals = line.split(":")
        parts = head.split()
        key = [int(x) for x in parts[2:6]]
        ctr = [int(x) for x in parts[6:10]]
        vals = [int(x) for x in vals.split()]
        nblk = (len(vals) + 7) // 8
        words = ctx.sitmo_blocks(key, ctr, nblk).reshape(-1)
        got = []
        for wd in words:
            got += [int(wd) & 0xFFFFFFFF, int(wd) >> 32]
        assert got[: len(vals)] == vals, head


def test_device_blocks_match_oracle_bulk(ctx):
    key = [0xABCDEF, 17, 3, 0]
    blocks = ctx.sitmo_blocks(key, [1 << 40, 9, 0, 0], 4096)
    for b in (0, 1, 777, 4095):
        assert np.array_equal(blocks[b], O.sitmo_block(key, [(1 << 40) + b, 9, 0, 0]))
