"""Python mirror of the learned pressure guess (fs_guess_* in include/fluid.h).

The network, its training and its use inside the projection run in
libfluidcuda.so; this module only moves arrays.  Data arguments are torch
CUDA tensors (f32, [B, H, W], contiguous) because the C entry points take
device pointers; numpy arrays are accepted and uploaded.

Normalisation (normalize_pair): with h the grid spacing of the stored fields
and sigma = RMS(h^2 div) per sample, the network sees h^2 div / sigma and the
solid mask, and is trained to output (p - mean p) / sigma.

Weights file ("FSGUESS" v1): 16-byte header {magic b"FSGUESS\\x01", u32
version = 1, u32 parameter count} then the f32 parameters, little-endian,
flattened layer by layer as w[c_out][c_in][3][3] then b[c_out].
"""
from __future__ import annotations

import ctypes as C
import struct
from pathlib import Path

import numpy as np

from . import _lib

WEIGHTS_MAGIC = b"FSGUESS\x01"


def _torch():
    import torch

    return torch


def _dev(x, torch):
    if isinstance(x, torch.Tensor):
        t = x.to(device="cuda", dtype=torch.float32)
    else:
        t = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32)).to("cuda")
    if t.dim() == 2:
        t = t[None]
    return t.contiguous()


def normalize_pair(div, mask, p, dx):
    """(div, mask, p) at grid spacing dx -> (div_n, mask, p_n, sigma)."""
    x = np.asarray(div, np.float64) * dx * dx
    sigma = float(np.sqrt(np.mean(x * x)))
    sigma = sigma if sigma > 0 else 1.0
    pn = (np.asarray(p, np.float64) - np.mean(p)) / sigma
    return (x / sigma).astype(np.float32), np.asarray(mask, np.float32), pn.astype(np.float32), sigma


class PressureGuess:
    """fs_guess handle: create, predict, train, save/load weights."""

    def __init__(self, device: int = 0, seed: int = 0):
        self._lib = _lib.load()
        h = C.c_void_p()
        _lib.check(self._lib.fs_guess_create(device, seed, C.byref(h)))
        self._h = h
        self.n_params = int(self._lib.fs_guess_num_params(h))

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            self._lib.fs_guess_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -------------------------------------------------------------- params
    def get_params(self) -> np.ndarray:
        out = np.empty(self.n_params, np.float32)
        _lib.check(self._lib.fs_guess_get_params(self._h, out.ctypes.data, self.n_params))
        return out

    def set_params(self, theta) -> None:
        t = np.ascontiguousarray(theta, np.float32)
        if t.size != self.n_params:
            raise ValueError(f"expected {self.n_params} parameters, got {t.size}")
        _lib.check(self._lib.fs_guess_set_params(self._h, t.ctypes.data, self.n_params))

    def save(self, path) -> None:
        th = self.get_params()
        with open(path, "wb") as f:
            f.write(WEIGHTS_MAGIC + struct.pack("<II", 1, th.size) + th.astype("<f4").tobytes())

    def load(self, path) -> None:
        b = Path(path).read_bytes()
        if b[:8] != WEIGHTS_MAGIC:
            raise ValueError(f"{path}: not an FSGUESS weights file")
        ver, n = struct.unpack("<II", b[8:16])
        if ver != 1 or n != self.n_params or len(b) != 16 + 4 * n:
            raise ValueError(f"{path}: version {ver}, {n} parameters (expected 1, {self.n_params})")
        self.set_params(np.frombuffer(b[16:], "<f4"))

    # ------------------------------------------------------------- compute
    def predict(self, div_n, mask):
        torch = _torch()
        d, m = _dev(div_n, torch), _dev(mask, torch)
        B, H, W = d.shape
        out = torch.empty_like(d)
        _lib.check(self._lib.fs_guess_predict(self._h, d.data_ptr(), m.data_ptr(), B, H, W, out.data_ptr()))
        return out

    def loss_grad(self, div_n, mask, target):
        torch = _torch()
        d, m, t = _dev(div_n, torch), _dev(mask, torch), _dev(target, torch)
        B, H, W = d.shape
        g = torch.empty(self.n_params, dtype=torch.float32, device="cuda")
        loss = C.c_double()
        _lib.check(self._lib.fs_guess_loss_grad(self._h, d.data_ptr(), m.data_ptr(), t.data_ptr(), B, H, W,
                                                C.byref(loss), g.data_ptr()))
        return loss.value, g

    def train_step(self, div_n, mask, target, lr: float, want_loss: bool = True):
        torch = _torch()
        d, m, t = _dev(div_n, torch), _dev(mask, torch), _dev(target, torch)
        B, H, W = d.shape
        loss = C.c_double()
        _lib.check(self._lib.fs_guess_train_step(self._h, d.data_ptr(), m.data_ptr(), t.data_ptr(), B, H, W,
                                                 C.c_float(lr), C.byref(loss) if want_loss else None))
        return loss.value if want_loss else None

    def set_loss(self, w_pressure: float = 1.0, w_residual: float = 0.0) -> None:
        """Loss = w_pressure * mean-free MSE + w_residual * mean (lap error)^2."""
        _lib.check(self._lib.fs_guess_set_loss(self._h, float(w_pressure), float(w_residual)))

    def sync(self):
        _lib.check(self._lib.fs_guess_sync(self._h))

    def launch_count(self) -> int:
        return int(self._lib.fs_guess_launch_count(self._h))


# ------------------------------------------------------------- pair files
def write_pair_file(path, div, mask, p, dx) -> None:
    lib = _lib.load()
    d = np.ascontiguousarray(div, np.float32)
    m = np.ascontiguousarray(mask, np.float32)
    q = np.ascontiguousarray(p, np.float32)
    ny, nx = d.shape
    _lib.check(lib.fs_write_pair_file(str(path).encode(), nx, ny, float(dx), d.ctypes.data, m.ctypes.data,
                                      q.ctypes.data))


def read_pair_file(path):
    """-> (div, mask, p, dx) as f32 [ny, nx] arrays."""
    lib = _lib.load()
    nx, ny, dx = C.c_int32(), C.c_int32(), C.c_double()
    _lib.check(lib.fs_read_pair_file(str(path).encode(), C.byref(nx), C.byref(ny), C.byref(dx), None, None, None))
    d = np.empty((ny.value, nx.value), np.float32)
    m = np.empty_like(d)
    q = np.empty_like(d)
    _lib.check(lib.fs_read_pair_file(str(path).encode(), C.byref(nx), C.byref(ny), C.byref(dx), d.ctypes.data,
                                     m.ctypes.data, q.ctypes.data))
    return d, m, q, dx.value
