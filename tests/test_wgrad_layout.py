"""Index arithmetic of the tensor-core weight-gradient kernel (k_wgrad_tc in
fluid-sim_gb300/csrc/fs_guess.cu), restated on the CPU.

The kernel computes dW[co][ci][tap] = sum_p G[p][co] X[p + s_tap][ci] as
D[m][n] = sum_k A[m][k] B[n][k] with K = pixels, rows m = tap * c_in + ci of
the shifted input (A) and n = co of the output gradient (B).  It stages both
from NHWC bf16 by transposing 8 pixels x 8 channels blocks with byte
permutes into the no-swizzle K-major core-matrix layout that
fs_tc_gemm_check verifies on the GPU (16-byte core-matrix rows, LBO = the
distance between the two K chunks of a step), with its 8-row groups 272
bytes apart (SBO) so that neighbouring threads' blocks sit on different
shared-memory banks.  Here: the byte-permute transpose, every staged block
inside its buffer, and the GEMM read back through the descriptor layout
equal to the direct correlation for every M-block grouping the network
uses, with partial pixel tiles and padding rows.
"""
from __future__ import annotations

import numpy as np
import pytest


def _byte_perm(a, b, sel):
    x = [(a >> (8 * i)) & 255 for i in range(4)] + [(b >> (8 * i)) & 255 for i in range(4)]
    return sum(x[(sel >> (4 * k)) & 7] << (8 * k) for k in range(4))


def _transpose8x8(words):
    o = [[0] * 4 for _ in range(8)]
    for j in range(4):
        for jp in range(4):
            a, b = words[2 * jp][j], words[2 * jp + 1][j]
            o[2 * j][jp] = _byte_perm(a, b, 0x5410)
            o[2 * j + 1][jp] = _byte_perm(a, b, 0x7632)
    return o


SBO, LBO = 272, 128  # bytes between 8-row groups, between the two K chunks of a step


def _kmaj_block(R, g, q):
    return (q >> 1) * ((R // 8) * SBO) + g * SBO + (q & 1) * 128


def _desc_offset(R, row, k):
    """Byte offset the MMA reads for element (row, k) of an operand of R rows:
    K step k // 16 (R / 8 groups of SBO bytes each), 8-row group at SBO,
    K chunk at LBO, 16-byte core-matrix rows."""
    return (k // 16) * ((R // 8) * SBO) + (row // 8) * SBO + ((k // 8) % 2) * LBO + (row % 8) * 16 + (k % 8) * 2


def test_transpose8x8():
    vals = np.random.default_rng(0).integers(0, 65536, size=(8, 8))
    words = [[int(vals[i, 2 * j]) | (int(vals[i, 2 * j + 1]) << 16) for j in range(4)] for i in range(8)]
    t = _transpose8x8(words)
    for c in range(8):
        for p in range(8):
            assert (t[c][p // 2] >> (16 * (p % 2))) & 0xFFFF == vals[p, c]


@pytest.mark.parametrize("cin,cout,nmb,B,H,W", [(16, 16, 2, 1, 3, 200), (32, 16, 3, 2, 4, 8),
                                                 (64, 128, 3, 1, 2, 128), (128, 64, 2, 1, 2, 64)])
def test_wgrad_staging_equals_correlation(cin, cout, nmb, B, H, W):
    """Tiles are segments of up to 128 pixels of one image row (the last one
    of a row partial); the three input rows around a tile (halo 1, periodic)
    are staged once, [3][130][c_in / 8] chunks, and every tap's block is read
    from that copy at the tap's shift."""
    rng = np.random.default_rng(cin + cout)
    X = rng.standard_normal((B, H, W, cin))
    G = rng.standard_normal((B, H, W, cout))
    kc_n, oc_n = cin // 8, cout // 8
    mrows = 9 * cin
    groups = (((mrows + 127) // 128) + nmb - 1) // nmb
    ntx = (W + 127) // 128
    D = np.zeros((groups * nmb * 128, cout))
    rows_a, ks = np.meshgrid(np.arange(128), np.arange(128), indexing="ij")
    RW = 130
    for gy in range(groups):
        mb0 = gy * nmb
        for t in range(B * H * ntx):
            xt, by = t % ntx, t // ntx
            y, b = by % H, by // H
            x0 = xt * 128
            xr = np.zeros((3, RW, cin))
            for r in range(3):
                for c in range(RW):
                    xr[r, c] = X[b, (y - 1 + r) % H, (x0 - 1 + c) % W]
            sb = np.zeros(8 * oc_n * SBO // 2)    # bf16 slots
            a_mb = 8 * 16 * SBO
            sa = np.zeros(nmb * a_mb // 2)
            for q in range(16):
                for oc in range(oc_n):
                    base = _kmaj_block(cout, oc, q) // 2
                    assert base + 64 <= sb.size
                    for i in range(8):
                        x = x0 + 8 * q + i
                        sb[base + np.arange(8) * 8 + i] = G[b, y, x, oc * 8:oc * 8 + 8] if x < W else 0
                for gl in range(nmb * 16):
                    gg = mb0 * 16 + gl
                    base = ((gl >> 4) * a_mb + _kmaj_block(128, gl & 15, q)) // 2
                    assert base + 64 <= sa.size
                    for i in range(8):
                        v = np.zeros(8)
                        if gg < 9 * kc_n:
                            tap, kc = gg // kc_n, gg % kc_n
                            col = 8 * q + (tap % 3) + i
                            assert 0 <= col < RW
                            v = xr[tap // 3, col, kc * 8:kc * 8 + 8]
                        sa[base + np.arange(8) * 8 + i] = v
            Bm = sb[_desc_offset(cout, *np.meshgrid(np.arange(cout), np.arange(128), indexing="ij")) // 2]
            for j in range(nmb):
                A = sa[(j * a_mb + _desc_offset(128, rows_a, ks)) // 2]
                D[(mb0 + j) * 128:(mb0 + j + 1) * 128] += A @ Bm.T
    Gf = G.reshape(-1, cout)
    ref = np.zeros((mrows, cout))
    for tap in range(9):
        Xs = np.roll(np.roll(X, -(tap // 3 - 1), axis=1), -(tap % 3 - 1), axis=2)
        ref[tap * cin:(tap + 1) * cin] = Xs.reshape(-1, cin).T @ Gf
    assert np.abs(D[:mrows] - ref).max() <= 1e-12 * np.abs(ref).max()
    assert not D[mrows:].any()
