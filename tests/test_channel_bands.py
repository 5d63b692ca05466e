"""Index arithmetic of the channel kernel (fs_channel.cu), restated on the CPU.

The kernel launches one 32x8 block grid over two bands: the rows the wall
slab can reach (every column), then the columns the fringe can reach outside
those rows.  For the channel geometry of the workloads at every size up to
8192^2: each band covers every face whose mask is >= 1e-7 (the kernel applies
the forcing where it is >= 1e-6), every launched index is in bounds, and each
cell of the union is visited exactly once (checked cell by cell up to 512^2).
"""
from __future__ import annotations

import math

import pytest

from conftest import load_package


def _band_of(x0, reach, h, n):
    lo = math.floor((x0 - reach) / h) - 1
    hi = math.ceil((x0 + reach) / h) + 1
    if hi - lo + 1 >= n:
        return 0, n
    return lo % n, hi - lo + 1


def _chi(d, half, w):
    return 0.5 * (1 - math.tanh((abs(d) - half) / w))


@pytest.mark.parametrize("n", [64, 128, 256, 512, 1024, 2048, 4096, 8192])
def test_channel_bands_cover_the_mask(n):
    L = 2 * math.pi
    h = L / n
    ch = load_package().workload.channel_geometry(L)
    w = 1.5 * h
    j0, nw = _band_of(ch["wall_y"], ch["wall_half"] + 8.5 * w, h, n)
    i0, nf = _band_of(ch["fringe_x"], ch["fringe_half"] + 8.5 * ch["fringe_ramp"], h, n)
    assert 0 < nw < n and 0 < nf < n
    rows = {(j0 + t) % n for t in range(nw)}
    cols = {(i0 + t) % n for t in range(nf)}

    def wrap(d):
        return d - L * math.floor(d / L + 0.5)

    for j in range(n):
        c = max(_chi(wrap((j + 0.5) * h - ch["wall_y"]), ch["wall_half"], w), _chi(wrap(j * h - ch["wall_y"]), ch["wall_half"], w))
        assert c < 1e-7 or j in rows
    for i in range(n):
        c = max(_chi(wrap(i * h - ch["fringe_x"]), ch["fringe_half"], ch["fringe_ramp"]),
                _chi(wrap((i + 0.5) * h - ch["fringe_x"]), ch["fringe_half"], ch["fringe_ramp"]))
        assert c < 1e-7 or i in cols
    if n > 512:
        return
    gxa = (n + 31) // 32
    na = gxa * ((nw + 7) // 8)
    gxb = (nf + 31) // 32
    nb = gxb * ((n - nw + 7) // 8)
    seen = {}
    for blk in range(na + nb):
        for ty in range(8):
            for tx in range(32):
                if blk < na:
                    i, t = (blk % gxa) * 32 + tx, (blk // gxa) * 8 + ty
                    if i >= n or t >= nw:
                        continue
                    j = (j0 + t) % n
                else:
                    k = blk - na
                    ti, t = (k % gxb) * 32 + tx, (k // gxb) * 8 + ty
                    if ti >= nf or t >= n - nw:
                        continue
                    i, j = (i0 + ti) % n, (j0 + nw + t) % n
                assert 0 <= i < n and 0 <= j < n
                seen[(i, j)] = seen.get((i, j), 0) + 1
    union = {(i, j) for j in rows for i in range(n)} | {(i, j) for i in cols for j in range(n)}
    assert set(seen) == union and max(seen.values()) == 1
