"""CPU restatement of the complex128 k-first row pass's line map
(lp_c128_lines.cuh, zline_kernel with Z_KINV on rows): for N <= 2048 a CTA
holds rows ky and N - ky (pair base b = 0 .. N/2) and evaluates their common
transfer-function table once.  The map must give every row of the grid to
exactly one live line, and both rows of a pair must have the same Ky**2 (the
table is built from the pair base), bit for bit in float64.
"""
import numpy as np
import pytest


def zgeo(n, lmin):
    """Lines per CTA and threads per line of ZGeo<N, LMIN> (8 points a thread)."""
    pt = 8
    tl = n // pt if n >= pt else 1
    l0 = 1 if tl >= 256 else 256 // tl
    return max(l0, lmin), tl


def kinv_lines(n):
    """(cta, slot, line, live, table_row) for every line slot of the pass."""
    tl = zgeo(n, 1)[1]
    pairs = tl <= 256
    L, _ = zgeo(n, 2 if pairs else 1)
    out = []
    if pairs:
        grid = (n // 2 + 1 + L // 2 - 1) // (L // 2)
        for blk in range(grid):
            for g in range(L):
                pb = blk * (L // 2) + g // 2
                second = g & 1
                line = n - pb if second else pb
                live = (1 <= pb < n // 2) if second else (pb <= n // 2)
                out.append((blk, g, line, live, pb))
    else:
        grid = (n + L - 1) // L
        for blk in range(grid):
            for g in range(L):
                line = blk * L + g
                out.append((blk, g, line, line < n, line))
    return out


@pytest.mark.parametrize("n", [2 ** k for k in range(1, 14)])
def test_every_row_once(n):
    rows = [line for _, _, line, live, _ in kinv_lines(n) if live]
    assert sorted(rows) == list(range(n))


@pytest.mark.parametrize("n", [2 ** k for k in range(1, 13)])
def test_pair_rows_share_ky_squared(n):
    val = 1.0 / (0.2 * 0.5)  # any grid step: the check is that the squares agree exactly
    h = (n + 1) // 2
    for _, _, line, live, trow in kinv_lines(n):
        if not live:
            continue
        fy_line = np.float64(line if line < h else line - n) * np.float64(val)
        fy_tab = np.float64(trow if trow < h else trow - n) * np.float64(val)
        assert fy_line * fy_line == fy_tab * fy_tab


def test_pairs_only_up_to_2048():
    # 4096 and 8192 keep one row per CTA (a pair would need 1024 or 2048 threads)
    for n, want in ((2048, True), (4096, False), (8192, False)):
        assert (zgeo(n, 1)[1] <= 256) == want
