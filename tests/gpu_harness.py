"""Helpers for the GPU parity tests: upload numpy images to CUDA memory with a
chosen row stride and byte offset, run an entry point through the C ABI, read
the result back and check that bytes outside the written region (the row
padding) were not touched."""
from __future__ import annotations

import numpy as np

CANARY = 0xA5


def device_image(torch, host: np.ndarray, offset: int = 0):
    """Copies a 2-D numpy image (rows x elements, any padding) to the GPU.
    `offset` bytes of misalignment are inserted before the first row."""
    es = host.dtype.itemsize
    nbytes = host.shape[0] * host.shape[1] * es
    buf = torch.empty(nbytes + offset + 64, dtype=torch.uint8, device="cuda")
    buf.fill_(0)
    view = buf[offset:offset + nbytes]
    view.copy_(torch.from_numpy(np.ascontiguousarray(host).view(np.uint8).reshape(-1)))
    return buf, view.data_ptr(), host.shape[1] * es


def device_output(torch, rows: int, row_elems: int, dtype, pad_elems: int = 0, offset: int = 0):
    es = np.dtype(dtype).itemsize
    stride = (row_elems + pad_elems) * es
    buf = torch.full((rows * stride + offset + 64,), CANARY, dtype=torch.uint8, device="cuda")
    return buf, buf.data_ptr() + offset, stride


def read_output(buf, rows: int, row_elems: int, dtype, stride: int, offset: int = 0):
    raw = buf.cpu().numpy()
    es = np.dtype(dtype).itemsize
    body = raw[offset:offset + rows * stride].reshape(rows, stride)
    out = body[:, : row_elems * es].copy().view(dtype)
    pad_ok = bool((body[:, row_elems * es:] == CANARY).all()) and bool((raw[:offset] == CANARY).all()) \
        and bool((raw[offset + rows * stride:] == CANARY).all())
    return out, pad_ok


def padded(rng, rows, row_elems, dtype, pad_elems=0, low=None, high=None):
    info = np.iinfo(dtype)
    lo = info.min if low is None else low
    hi = info.max if high is None else high
    return rng.integers(lo, int(hi) + 1, (rows, row_elems + pad_elems), dtype=dtype)


def pyr_sizes(w, h, levels):
    out = []
    for _ in range(levels):
        w, h = (w + 1) // 2, (h + 1) // 2
        out.append((w, h))
    return out


_CUDART = None


def _cudart():
    """The CUDA runtime through ctypes (raw device pointers that no tensor owns)."""
    import ctypes
    import glob
    import os

    global _CUDART
    if _CUDART is None:
        import torch

        cands = glob.glob(os.path.join(os.path.dirname(torch.__file__), "lib", "libcudart.so*"))
        cands += glob.glob("/usr/local/cuda/lib64/libcudart.so*")
        for c in cands:
            try:
                _CUDART = ctypes.CDLL(c)
                break
            except OSError:
                continue
        if _CUDART is None:
            _CUDART = ctypes.CDLL("libcudart.so")
        _CUDART.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    return _CUDART


def copy_from_device(ptr: int, nbytes: int) -> np.ndarray:
    """Device bytes at a raw pointer -> host uint8 array (synchronous)."""
    import ctypes

    out = np.empty(nbytes, np.uint8)
    err = _cudart().cudaMemcpy(ctypes.c_void_p(out.ctypes.data), ctypes.c_void_p(ptr), ctypes.c_size_t(nbytes), 2)
    assert err == 0, err
    return out


def read_strided(ptr: int, rows: int, row_bytes: int, stride: int) -> np.ndarray:
    """rows x row_bytes bytes starting at a device pointer, rows `stride` apart."""
    raw = copy_from_device(ptr, (rows - 1) * stride + row_bytes)
    return np.stack([raw[r * stride: r * stride + row_bytes] for r in range(rows)]) if rows else \
        np.zeros((0, row_bytes), np.uint8)
