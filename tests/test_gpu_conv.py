"""The tensor-core 3x3 convolution (fs_conv3x3_bf16) and its GEMM self-check.

Inputs and weights are drawn bf16-exact, so the only rounding on the device
side is the f32 accumulation order and the final bf16 store; the reference is
a float64 periodic convolution (numpy, np.roll per tap).  Tolerance: 1e-2
relative to the output's largest magnitude (bf16 keeps 8 significant bits).
"""
from __future__ import annotations

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

PAIRS = [(16, 16), (16, 32), (32, 16), (32, 64), (64, 32), (64, 128), (128, 64)]


def _bf16_exact(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(torch.bfloat16).float().numpy()


def pack_weights(w):
    """[co][ci][3][3] -> [ky*3+kx][ci/8][co][ci%8] (the B operand layout)."""
    co, ci = w.shape[:2]
    t = w.transpose(2, 3, 1, 0).reshape(9, ci // 8, 8, co)
    return np.ascontiguousarray(t.transpose(0, 1, 3, 2))


def conv_ref(x, w, b, relu):
    out = np.zeros(x.shape[:3] + (w.shape[0],))
    for ky in range(3):
        for kx in range(3):
            xs = np.roll(x, shift=(-(ky - 1), -(kx - 1)), axis=(1, 2))
            out += np.einsum("bhwc,oc->bhwo", xs, w[:, :, ky, kx].astype(np.float64))
    out += b
    return np.maximum(out, 0.0) if relu else out


@pytest.fixture(scope="module")
def lib(fs):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return fs._lib.load()


def _run_conv(lib, fs, x, w, b, epi):
    dev = torch.device("cuda")
    B, H, W, ci = x.shape
    co = w.shape[0]
    xin = torch.from_numpy(x).to(dev).to(torch.bfloat16).contiguous()
    wp = torch.from_numpy(pack_weights(w)).to(dev).to(torch.bfloat16).contiguous()
    bias = torch.from_numpy(b.astype(np.float32)).to(dev)
    if epi == 2:
        out = torch.zeros((B, H, W), dtype=torch.float32, device=dev)
    else:
        out = torch.zeros((B, H, W, co), dtype=torch.bfloat16, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    st = lib.fs_conv3x3_bf16(xin.data_ptr(), wp.data_ptr(), bias.data_ptr(), out.data_ptr(), B, H, W, ci, co, epi,
                             err.data_ptr(), torch.cuda.current_stream().cuda_stream)
    fs._lib.check(st)
    torch.cuda.synchronize()
    assert int(err.item()) == 0, "tensor-core completion wait timed out"
    return out.float().cpu().numpy()


@pytest.mark.parametrize("n", [16, 64])
@pytest.mark.parametrize("k", [16, 64])
def test_gemm_check(lib, fs, n, k):
    rng = np.random.default_rng(n * 100 + k)
    a = _bf16_exact(rng.standard_normal((128, k)))
    b = _bf16_exact(rng.standard_normal((n, k)))
    dev = torch.device("cuda")
    ta = torch.from_numpy(a).to(dev).to(torch.bfloat16).contiguous()
    tb = torch.from_numpy(b).to(dev).to(torch.bfloat16).contiguous()
    d = torch.zeros((128, n), dtype=torch.float32, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    fs._lib.check(lib.fs_tc_gemm_check(ta.data_ptr(), tb.data_ptr(), d.data_ptr(), n, k, err.data_ptr(),
                                       torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    ref = a.astype(np.float64) @ b.astype(np.float64).T
    np.testing.assert_allclose(d.cpu().numpy(), ref, rtol=1e-5, atol=1e-4)


@pytest.mark.parametrize("ci,co", PAIRS)
@pytest.mark.parametrize("shape", [(2, 5, 40), (1, 9, 293)])
def test_conv_matches_numpy(lib, fs, ci, co, shape):
    B, H, W = shape
    rng = np.random.default_rng(ci * 1000 + co + H)
    x = _bf16_exact(rng.standard_normal((B, H, W, ci)))
    w = _bf16_exact(rng.standard_normal((co, ci, 3, 3)) / np.sqrt(9 * ci))
    b = rng.standard_normal(co).astype(np.float32) * 0.1
    got = _run_conv(lib, fs, x, w, b, 1)
    ref = conv_ref(x.astype(np.float64), w, b, True)
    np.testing.assert_allclose(got, ref, rtol=1e-2, atol=1e-2 * np.abs(ref).max())


def test_conv_linear_and_channel0(lib, fs):
    rng = np.random.default_rng(7)
    x = _bf16_exact(rng.standard_normal((1, 16, 130, 16)))
    w = _bf16_exact(rng.standard_normal((16, 16, 3, 3)) / 12.0)
    b = rng.standard_normal(16).astype(np.float32)
    ref = conv_ref(x.astype(np.float64), w, b, False)
    got = _run_conv(lib, fs, x, w, b, 0)
    np.testing.assert_allclose(got, ref, rtol=1e-2, atol=1e-2 * np.abs(ref).max())
    got0 = _run_conv(lib, fs, x, w, b, 2)  # f32 channel 0, no bf16 rounding of the output
    np.testing.assert_allclose(got0, ref[..., 0], rtol=1e-4, atol=1e-4 * np.abs(ref).max())


def test_conv_rejects_bad_arguments(lib, fs):
    st = lib.fs_conv3x3_bf16(None, None, None, None, 1, 8, 8, 16, 16, 1, None, None)
    assert st == 1
    dev = torch.device("cuda")
    t = torch.zeros(4096, dtype=torch.bfloat16, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    st = lib.fs_conv3x3_bf16(t.data_ptr(), t.data_ptr(), t.data_ptr(), t.data_ptr(), 1, 8, 8, 16, 48, 1,
                             err.data_ptr(), None)
    assert st == 6  # FS_ERR_UNSUPPORTED
