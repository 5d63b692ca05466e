"""The CPU restatement of the pressure-guess network (oracle/guess_oracle.py)
and the training-pair file format -- no GPU needed.

* the oracle's analytic gradient against central finite differences along
  random directions (float64, relative error <= 1e-6);
* the parameter count and layout the C ABI reports for the same network;
* FSPAIR files written and read back through the C ABI (host code only),
  and a corrupted header rejected.
"""
from __future__ import annotations

import numpy as np
import pytest

import guess_oracle as G


def _problem(seed=0, B=1, H=16, W=16):
    rng = np.random.default_rng(seed)
    theta = G.init_params(seed).astype(np.float64)
    theta += 0.05 * rng.standard_normal(theta.shape)  # non-zero biases, no dead layers
    div = rng.standard_normal((B, H, W))
    mask = (rng.random((B, H, W)) > 0.7).astype(np.float64)
    tgt = rng.standard_normal((B, H, W))
    return rng, theta, div, mask, tgt


def test_layer_table_and_count():
    assert [l[1:3] for l in G.LAYERS] == [(16, 16), (16, 16), (16, 32), (32, 64), (64, 128), (128, 64),
                                          (64, 32), (32, 16), (16, 16), (16, 16)]
    assert G.num_params() == sum(ci * co * 9 + co for _, ci, co, _ in G.LAYERS)


@pytest.mark.parametrize("seed,w", [(0, (1.0, 0.0)), (1, (1.0, 0.0)), (2, (0.3, 1.0))])
def test_gradient_matches_finite_differences(seed, w):
    """One random direction per parameter block (each layer's w, then b):
    a direction over all ~200k parameters at once moves enough ReLUs across
    their kink for the central difference itself to be off."""
    rng, theta, div, mask, tgt = _problem(seed, B=2 if seed else 1)
    L, g, _ = G.loss_grad(theta, div, mask, tgt, w_p=w[0], w_r=w[1])
    assert np.isfinite(L) and L > 0
    eps = 1e-6
    k = 0
    for name, ci, co, _ in G.LAYERS:
        for size in (ci * co * 9, co):
            d = np.zeros_like(theta)
            d[k:k + size] = rng.standard_normal(size)
            k += size
            lp = G.loss_grad(theta + eps * d, div, mask, tgt, w_p=w[0], w_r=w[1])[0]
            lm = G.loss_grad(theta - eps * d, div, mask, tgt, w_p=w[0], w_r=w[1])[0]
            fd = (lp - lm) / (2 * eps)
            assert abs(fd - g @ d) <= 1e-6 * max(1.0, abs(fd)), (name, size, fd, g @ d)


def test_padded_input_channels_get_no_gradient():
    _, theta, div, mask, tgt = _problem(3)
    _, g, _ = G.loss_grad(theta, div, mask, tgt)
    gA = g[:16 * 16 * 9].reshape(16, 16, 3, 3)
    assert np.all(gA[:, 2:] == 0.0)


def test_adam_first_step_is_sign_like():
    th = np.zeros(4)
    g = np.array([1.0, -2.0, 0.0, 1e-3])
    new, m, v = G.adam(th, g, np.zeros(4), np.zeros(4), 1, 0.01)
    np.testing.assert_allclose(new[[0, 1, 3]], [-0.01, 0.01, -0.01], rtol=1e-4)
    assert new[2] == 0.0


def test_pair_file_round_trip(fs, tmp_path):
    lib = fs._lib.load()
    rng = np.random.default_rng(2)
    d, m, p = (rng.standard_normal((24, 40)).astype(np.float32) for _ in range(3))
    path = tmp_path / "pair.fspair"
    fs.write_pair_file(path, d, m, p, 0.125)
    raw = path.read_bytes()
    assert raw[:8] == b"FSPAIR\x00\x01" and len(raw) == 40 + 3 * 24 * 40 * 4
    d2, m2, p2, dx = fs.read_pair_file(path)
    assert dx == 0.125
    for a, b in ((d, d2), (m, m2), (p, p2)):
        np.testing.assert_array_equal(a, b)
    bad = tmp_path / "bad.fspair"
    bad.write_bytes(b"NOTAPAIR" + raw[8:])
    with pytest.raises(fs.FluidError):
        fs.read_pair_file(bad)
    trunc = tmp_path / "trunc.fspair"
    trunc.write_bytes(raw[:100])
    with pytest.raises(fs.FluidError):
        fs.read_pair_file(trunc)
    assert lib.fs_write_pair_file(str(path).encode(), 0, 4, 1.0, None, None, None) == 1


def test_normalize_pair_is_scale_free(fs):
    rng = np.random.default_rng(4)
    d, m, p = rng.standard_normal((3, 16, 16))
    a = fs.normalize_pair(d, m, p, 0.1)
    b = fs.normalize_pair(5 * d, m, 5 * p + 3.0, 0.1)
    np.testing.assert_allclose(a[0], b[0], rtol=1e-6)
    np.testing.assert_allclose(a[2], b[2], rtol=1e-5, atol=1e-6)
