"""The traversal's closed-form ascend (svo_trace.cuh: svo_trace_run) against the
one-level-at-a-time climb it replaced, exhaustively on the CPU: for every
extent L = 6..14, every level, every cell and both step directions inside the
cube, the level found from the highest differing coordinate bit and the
first-level-of-size table equals the climb's."""
from __future__ import annotations


def level_log2(L: int, li: int) -> int:
    return 0 if li == 0 else li + 1 if li <= 2 else min(2 * li - 1, L - 1)


def n_levels(L: int) -> int:
    n = 4
    while level_log2(L, n - 1) < L - 1:
        n += 1
    return n


def climb(L: int, NL: int, li: int, g: int, prev: int, cur: int) -> int:
    li_u, g_u = li, g
    while li_u < NL - 1:
        gp = level_log2(L, li_u + 1)
        sh = gp - g_u
        if (prev >> sh) == (cur >> sh):
            break
        prev >>= sh
        cur >>= sh
        li_u += 1
        g_u = gp
    return li_u


def first_level_table(L: int, NL: int, size: int = 48) -> list[int]:
    out = []
    for k in range(size):
        f = NL
        if k <= L - 1:
            for li in range(NL):
                if level_log2(L, li) >= k:
                    f = li
                    break
        out.append(f)
    return out


def test_closed_form_ascend_equals_the_climb():
    checked = 0
    for L in range(6, 15):
        NL = n_levels(L)
        first = first_level_table(L, NL)
        for li in range(NL):
            g = level_log2(L, li)
            cells = 1 << (L - g)
            for prev in range(cells):
                for cur in (prev - 1, prev + 1):
                    if not 0 <= cur < cells:
                        continue
                    diff = prev ^ cur
                    need = g + diff.bit_length()
                    closed = min(NL - 1, max(li, first[min(need, 47)] - 1))
                    assert closed == climb(L, NL, li, g, prev, cur), (L, li, prev, cur)
                    checked += 1
    assert checked > 90000
