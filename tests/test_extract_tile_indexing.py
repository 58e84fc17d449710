"""Index arithmetic of the extraction row pass's output tile, on the CPU.

k_extract_rows stores the kx band through a shared-memory tile: row pair tr
of the CTA (lane j of its transform) writes column c of each round at tile
word c (P + 1) + tr, and the CTA's threads drain word c (P + 1) + p to float4
(cb + c) H/2 + p of the CTA's column segments.  This restates that
arithmetic for every supported hologram size and band width. It checks
that every (column, row pair) word is written once and lands in its own
column segment, that all accesses stay inside the tile and the output, that
a quarter-warp's 16-byte accesses hit distinct bank groups, and that the
CTA's shared memory fits the 227 KB per-CTA limit.
"""
from __future__ import annotations

import pytest


def _cfg(H):
    E = 64 if H >= 2048 else 32 if H >= 512 else 16 if H >= 128 else 8  # points per lane
    T = H // E
    G = 32 // T
    P = 8 * G
    stride = H + E + 1
    CB = 1024 // P
    smem = P * stride * 8 + CB * (P + 1) * 16
    return E, T, G, P, CB, smem


def _banks(word16):
    b = (word16 * 4) % 32
    return {b, b + 1, b + 2, b + 3}


@pytest.mark.parametrize("H", [256, 512, 1024, 2048])
def test_tile_fill_and_drain(H):
    E, T, G, P, CB, smem = _cfg(H)
    assert smem + 8 * 8 <= 227 * 1024  # plus the row pass's static mbarriers
    NT = 256
    assert NT // T == P  # one row pair per transform, P transforms per CTA
    for F in (64, 128, 256, 512):
        if F > H:
            continue
        placed = {}
        for cb in range(0, F, CB):
            nc = min(CB, F - cb)
            tile = {}
            # fill: each transform's lanes, in lane order, 16-byte words
            for tr in range(P):
                for c0 in range(0, nc, T):
                    quarter = []
                    for j in range(T):
                        c = c0 + j
                        if c >= nc:
                            continue
                        w = c * (P + 1) + tr
                        assert 0 <= w < CB * (P + 1)
                        assert w not in tile
                        tile[w] = (cb + c, tr)
                        quarter.append(w)
                        if len(quarter) == 8:
                            used = [_banks(x) for x in quarter]
                            assert len(set().union(*used)) == 32  # 8 lanes, 8 distinct bank groups
                            quarter = []
            assert len(tile) == nc * P
            # drain: consecutive threads take consecutive row pairs of a column
            for i0 in range(0, nc * P, NT):
                for q0 in range(i0, min(i0 + NT, nc * P), 8):
                    ws = [(i // P) * (P + 1) + i % P for i in range(q0, min(q0 + 8, nc * P))]
                    if len(ws) == 8:
                        assert len(set().union(*[_banks(x) for x in ws])) == 32
                for i in range(i0, min(i0 + NT, nc * P)):
                    c, p = i // P, i % P
                    w = c * (P + 1) + p
                    col, pair = tile[w]
                    assert (col, pair) == (cb + c, p)
                    dst = (cb + c) * (H // 2) + p  # float4 index from the CTA's segment base
                    assert dst not in placed
                    placed[dst] = (col, pair)
        assert len(placed) == F * P
        # the CTA's segment of column c holds its P row pairs in order
        for (col, pair) in placed.values():
            assert 0 <= col < F and 0 <= pair < P
        assert max(placed) < F * (H // 2)
