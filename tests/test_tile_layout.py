"""CPU checks of the multigrid tile kernels' index arithmetic (fs_multigrid.cu).

The fused down / up kernels stage a tile's region into shared memory by TMA
boxes whose first column must sit on a 16-byte boundary, then sweep, restrict
and prolong by fixed offsets.  A wrong constant would read or write outside a
shared array or outside the grid.  These tests restate the layout constants
(TileBox, CoarseBox) and the kernels' loops over cells, for every template
instance the library builds (tiles of 16, 32 and 64 cells, pre / post sweeps
1..3), and check that every access stays inside its array, that each
red-black half-sweep updates exactly the cells of its colour, and that the
2x2-block prolongation gives every region cell the coarse values and weights
of the per-cell formula (multigrid.js:99-131).
"""
from __future__ import annotations

import numpy as np
import pytest

NTH = 256  # threads of a tile kernel
TILES = (16, 32, 64)


def tilebox(T, H):
    R = T + 2 * H
    LP = (H + 3) & ~3
    OX = LP - H
    W = (LP + T + H + 3) & ~3
    N = W * R
    NA = (N + 31) & ~31
    return R, LP, OX, W, N, NA


def coarsebox(T, H):
    RC = (T + 2 * H) // 2 + 2
    LPC = (H // 2 + 1 + 3) & ~3
    OC = LPC - (H // 2 + 1)
    WC = (OC + RC + 3) & ~3
    NC = (WC * RC + 31) & ~31
    return RC, LPC, OC, WC, NC


def sweep(R, W, OX, par0, c):
    """rb_half_tile: the (li, lj) each thread updates and every offset it reads"""
    NI = R - 2
    NCH = NTH // NI
    assert NCH >= 1 and W % 2 == 0
    CH = ((NI + NCH - 1) // NCH + 1) & ~1
    offs, upd = [], []
    for tid in range(NTH):
        chunk, m = divmod(tid, NI)
        if chunk >= NCH:
            continue
        li = 1 + m
        lj = 1 + chunk * CH
        lend = min(lj + CH, R - 1)
        lj += (par0 + li + lj + c) & 1
        if lj >= lend:
            continue
        p = lj * W + OX + li
        offs.append(p - W)
        while lj < lend:
            offs += [p + W, p, p - 1, p + 1]
            upd.append((li, lj))
            lj += 2
            p += 2 * W
    return offs, upd


@pytest.mark.parametrize("T", TILES)
@pytest.mark.parametrize("pre", (1, 2, 3))
def test_down_kernel_layout(T, pre):
    H = 2 * pre + 1
    R, LP, OX, W, N, NA = tilebox(T, H)
    assert LP % 4 == 0 and W % 4 == 0 and OX + R <= W and W <= 256 and R <= 256 and NA % 32 == 0
    for par0 in (0, 1):
        for c in (0, 1):
            offs, upd = sweep(R, W, OX, par0, c)
            assert 0 <= min(offs) and max(offs) < N
            want = {(li, lj) for li in range(1, R - 1) for lj in range(1, R - 1) if (par0 + li + lj) & 1 == c}
            assert len(upd) == len(set(upd)) and set(upd) == want
    # tile write-back (float4) and the residual's 2x2 blocks (float2 rows)
    for y in range(T):
        o = (H + y) * W + LP
        assert o % 4 == 0 and o + T - 1 < N
    for cj in range(T // 2):
        for ci in range(T // 2):
            off = (H + 2 * cj) * W + LP + 2 * ci
            assert off % 2 == 0
            for d in (0, 1, W, W + 1, -W, -W + 1, 2 * W, 2 * W + 1, -1, 2, W - 1, W + 2):
                assert 0 <= off + d < N


@pytest.mark.parametrize("T", TILES)
@pytest.mark.parametrize("post", (1, 2, 3))
def test_up_kernel_layout(T, post):
    H = 2 * post
    R, LP, OX, W, N, NA = tilebox(T, H)
    RC, LPC, OC, WC, NC = coarsebox(T, H)
    assert LPC % 4 == 0 and WC % 4 == 0 and OC + RC <= WC and WC * RC <= NC
    for par0 in (0, 1):
        for c in (0, 1):
            offs, upd = sweep(R, W, OX, par0, c)
            assert 0 <= min(offs) and max(offs) < N
            assert len(upd) == len(set(upd)) == sum(
                1 for li in range(1, R - 1) for lj in range(1, R - 1) if (par0 + li + lj) & 1 == c)
    # prolongation by even-aligned 2x2 fine blocks, a thread walking one
    # column of blocks down a chunk of block rows: each region cell once,
    # with the coarse column / row and the weights of the per-cell formula,
    # every float2 aligned and every coarse load inside the block
    NBC = R // 2
    NCK = 256 // NBC
    CL = (NBC + NCK - 1) // NCK
    assert NCK >= 1 and OX % 2 == 0 and W % 2 == 0
    seen = set()
    for tid in range(256):
        chunk, e = divmod(tid, NBC)
        for d in range(chunk * CL, min(chunk * CL + CL, NBC)) if chunk < NCK else ():
            for r in range(3):
                for q in range(3):
                    assert 0 <= (d + r) * WC + OC + e + q < WC * RC and OC + e + q < WC
            top = 2 * d * W + OX + 2 * e
            assert top % 2 == 0
            # (offset, first coarse column, first coarse row, fx, fy)
            for o, cx, cy, fx, fy in ((top, e, d, 0.75, 0.75), (top + 1, e + 1, d, 0.25, 0.75),
                                      (top + W, e, d + 1, 0.75, 0.25), (top + W + 1, e + 1, d + 1, 0.25, 0.25)):
                lj, rem = divmod(o, W)
                li = rem - OX
                assert 0 <= li < R and 0 <= lj < R and o not in seen
                assert (li + 1) >> 1 == cx and (lj + 1) >> 1 == cy
                assert fx == (0.25 if li & 1 else 0.75) and fy == (0.25 if lj & 1 else 0.75)
                seen.add(o)
    assert len(seen) == R * R
    for y in range(T):
        o = (H + y) * W + LP
        assert o % 4 == 0 and o + T - 1 < N


def tile_fits(t, n):
    """the side rule of mg_tile / tile_for_class: T <= n / 2 (16 always)"""
    return t == 16 or 2 * t <= n


@pytest.mark.parametrize("n", (2048, 1024, 528, 384, 200, 192, 132, 128, 72, 70, 68, 66))
def test_tma_boxes_and_wrapped_staging(n):
    """For every tile of every side a level may use: on a level with tensor
    maps (n % 4 == 0, the box no larger than the grid) every tile's boxes --
    the region's and the up kernel's coarse block -- start on a multiple of 4
    columns (16 bytes), also where they cross the grid's edge, and every cell
    of a box outside the grid (zero-filled by the copy, then replaced by its
    periodic image) needs at most one wrap; a tile inside the grid writes back
    in aligned float4 rows; the wrapped staging of levels without tensor maps
    needs at most one wrap."""
    for T in TILES:
        if not tile_fits(T, n):
            continue
        k = (n + T - 1) // T
        for H in (3, 5, 7, 2, 4, 6):
            R, LP, OX, W, N, NA = tilebox(T, H)
            nc = n // 2
            for by in range(k):
                for bx in range(k):
                    i0, j0 = bx * T, by * T
                    gi0, gj0 = i0 - H, j0 - H
                    assert -n <= gi0 and gi0 + R - 1 < 2 * n and -n <= gj0 and gj0 + R - 1 < 2 * n
                    tma = n % 4 == 0 and W <= n and R <= n
                    if tma:
                        bx0 = i0 - LP
                        assert bx0 % 4 == 0 and gi0 - bx0 == OX
                        assert -n < bx0 and bx0 + W - 1 < 2 * n and -n < gj0 and gj0 + R - 1 < 2 * n
                        if i0 + T <= n and j0 + T <= n:
                            assert (j0 * n + i0) % 4 == 0 and T % 4 == 0
                    if H % 2 == 0:  # up kernel: the coarse block
                        RC, LPC, OC, WC, NC = coarsebox(T, H)
                        cgi0, cgj0 = (gi0 >> 1) - 1, (gj0 >> 1) - 1
                        assert -nc <= cgi0 and cgi0 + RC - 1 < 2 * nc and -nc <= cgj0 and cgj0 + RC - 1 < 2 * nc
                        if tma and nc % 4 == 0 and WC <= nc and RC <= nc:
                            cbx = cgi0 - OC
                            assert cbx % 4 == 0 and -nc < cbx and cbx + WC - 1 < 2 * nc


def _ring(pitch, rows, bx, by, n):
    """ring_cells / ring_cell (fs_multigrid.cu) restated: the (row, column)
    of every box cell outside the grid, in the kernel's order."""
    cl, cr = max(0, -bx), max(0, bx + pitch - n)
    rb, rt = max(0, -by), max(0, by + rows - n)
    cells = []
    for k in range((rb + rt) * pitch + (rows - rb - rt) * (cl + cr)):
        nrow = (rb + rt) * pitch
        if k < nrow:
            q, c = divmod(k, pitch)
            r = q if q < rb else rows - rt + (q - rb)
        else:
            q, m = divmod(k - nrow, cl + cr)
            r, c = rb + q, (m if m < cl else pitch - cr + (m - cl))
        cells.append((r, c))
    return cells


def _wrap_box_ring(dst, pitch, rows, src, bx, by, n):
    w1 = lambda i: i + n if i < 0 else (i - n if i >= n else i)  # noqa: E731
    cells = _ring(pitch, rows, bx, by, n)
    assert len(set(cells)) == len(cells)
    for r, c in cells:
        assert 0 <= r < rows and 0 <= c < pitch
        dst[r * pitch + c] = src[w1(by + r) * n + w1(bx + c)]


@pytest.mark.parametrize("n,T,H", [(64, 16, 5), (68, 16, 4), (72, 32, 4), (132, 64, 5), (200, 16, 6), (128, 64, 4)])
def test_edge_box_fixup_equals_periodic_staging(n, T, H):
    """A box copied with zero fill outside the grid and then fixed up holds,
    in every cell, the periodic image the wrapped staging would read."""
    R, LP, OX, W, N, NA = tilebox(T, H)
    if W > n or R > n:
        pytest.skip("no tensor map for this level")
    src = np.arange(n * n, dtype=np.float64) + 1.0
    k = (n + T - 1) // T
    for tby in range(k):
        for tbx in range(k):
            bx, by = tbx * T - LP, tby * T - H
            box = np.zeros(W * R)
            for r in range(R):
                for c in range(W):
                    gx, gy = bx + c, by + r
                    if 0 <= gx < n and 0 <= gy < n:
                        box[r * W + c] = src[gy * n + gx]
            _wrap_box_ring(box, W, R, src, bx, by, n)
            want = np.array([src[((by + r) % n) * n + (bx + c) % n] for r in range(R) for c in range(W)])
            assert np.array_equal(box, want), (tbx, tby)
