"""ctypes front-end of the C oracle (kcv_oracle.c).

TEST INFRASTRUCTURE ONLY: the product library never imports this module.  It is
used by tests/ as the parity checker, by ``__graft_entry__.smoke()`` as the
checker of the smoke run, and by ``bench.py`` for the CPU baseline
("port", since the reference itself is AArch64-only C++ that neither this
container nor the GPU machine can build from its sources).

Images are 2-D numpy arrays whose first axis is the row; row strides are taken
from ``array.strides[0]`` so padded layouts (stride > width*channels*elem) are
passed through exactly like the C API's ``src_stride`` / ``dst_stride``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libkcv_oracle.so")

OK, NOT_IMPLEMENTED, NULL_POINTER, RANGE, ALLOCATION, ALIGNMENT = 0, 1, 2, 3, 4, 5
CONSTANT, REPLICATE, REFLECT, WRAP, REVERSE, TRANSPARENT, NONE = range(7)
FIXED_BORDERS = (REPLICATE, REFLECT, WRAP, REVERSE)

_lib = None


def build(force: bool = False) -> str:
    """Compiles the oracle with the recipe in oracle/Makefile."""
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(
        os.path.getmtime(os.path.join(HERE, f)) for f in ("kcv_oracle.c", "kcv_oracle.h", "Makefile")
    ):
        subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB_PATH)
        sz, vp, f, i = ctypes.c_size_t, ctypes.c_void_p, ctypes.c_float, ctypes.c_int
        _lib.ko_gaussian_half_kernel.argtypes = [vp, sz, f]
        _lib.ko_border_map.argtypes = [ctypes.c_long, ctypes.c_long, i]
        _lib.ko_border_map.restype = ctypes.c_long
        _lib.ko_border_table.argtypes = [i, ctypes.c_long, i, vp]
        _lib.ko_gaussian_blur_u8.argtypes = [vp, sz, vp, sz, sz, sz, sz, sz, sz, f, f, i, i, i, i]
        for name in ("ko_separable_filter_2d_u8", "ko_separable_filter_2d_u16"):
            getattr(_lib, name).argtypes = [vp, sz, vp, sz, sz, sz, sz, vp, sz, vp, sz, i, i, i, i]
        _lib.ko_separable_filter_2d_s16.argtypes = [vp, sz, vp, sz, sz, sz, sz, vp, sz, vp, sz, i, i, i]
        _lib.ko_blur_and_downsample_u8.argtypes = [vp, sz, sz, sz, vp, sz, sz, i, i, i, i]
        for name in ("ko_sobel_3x3_horizontal_s16_u8", "ko_sobel_3x3_vertical_s16_u8"):
            getattr(_lib, name).argtypes = [vp, sz, vp, sz, sz, sz, sz, i]
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


def _stride(a):
    return 0 if a is None else int(a.strides[0])


def half_kernel(ksize: int, sigma: float):
    """Returns the half kernel (list of ksize//2+1 ints) or None for 'copy'."""
    half = np.zeros(128, np.uint8)
    ok = lib().ko_gaussian_half_kernel(half.ctypes.data, ksize // 2 + 1, float(sigma))
    return [int(v) for v in half[: ksize // 2 + 1]] if ok else None


def border_map(i: int, n: int, border: int) -> int:
    return lib().ko_border_map(i, n, border)


def border_table(ksize: int, n: int, border: int) -> np.ndarray:
    out = np.zeros((n, ksize), np.int64)
    lib().ko_border_table(ksize, n, border, out.ctypes.data)
    return out


def _out_like(src, width, height, channels, dtype, out_w=None, out_h=None):
    ow = width if out_w is None else out_w
    oh = height if out_h is None else out_h
    return np.zeros((max(oh, 1), max(ow * channels, 1)), dtype)


def gaussian_blur_u8(src, width, height, channels, ksize, sigma, border, *, ext=False,
                     border_value=0, nthreads=1, dst=None, ksize_y=None, sigma_y=None):
    if dst is None and src is not None:
        dst = _out_like(src, width, height, channels, np.uint8)
    err = lib().ko_gaussian_blur_u8(
        _ptr(src), _stride(src), _ptr(dst), _stride(dst), width, height, channels, ksize,
        ksize if ksize_y is None else ksize_y, float(sigma),
        float(sigma if sigma_y is None else sigma_y), border, int(ext), int(border_value), nthreads)
    return err, dst


def separable_filter_2d(src, width, height, channels, kernel_x, kernel_y, border, *, ext=False,
                        border_value=0, nthreads=1, dst=None, kw=None, kh=None):
    dtype = src.dtype if src is not None else np.dtype(kernel_x.dtype)
    if dst is None and src is not None:
        dst = _out_like(src, width, height, channels, dtype)
    kx = None if kernel_x is None else np.ascontiguousarray(kernel_x, dtype)
    ky = None if kernel_y is None else np.ascontiguousarray(kernel_y, dtype)
    kw = (len(kx) if kx is not None else 5) if kw is None else kw
    kh = (len(ky) if ky is not None else 5) if kh is None else kh
    if dtype == np.uint8:
        err = lib().ko_separable_filter_2d_u8(_ptr(src), _stride(src), _ptr(dst), _stride(dst), width, height,
                                              channels, _ptr(kx), kw, _ptr(ky), kh, border, int(ext),
                                              int(border_value), nthreads)
    elif dtype == np.uint16:
        err = lib().ko_separable_filter_2d_u16(_ptr(src), _stride(src), _ptr(dst), _stride(dst), width, height,
                                               channels, _ptr(kx), kw, _ptr(ky), kh, border, int(ext),
                                               int(border_value), nthreads)
    elif dtype == np.int16:
        err = lib().ko_separable_filter_2d_s16(_ptr(src), _stride(src), _ptr(dst), _stride(dst), width, height,
                                               channels, _ptr(kx), kw, _ptr(ky), kh, border, int(border_value),
                                               nthreads)
    else:
        raise TypeError(dtype)
    return err, dst


def blur_and_downsample_u8(src, width, height, channels, border, *, ext=False, border_value=0,
                           nthreads=1, dst=None):
    if dst is None and src is not None:
        dst = _out_like(src, width, height, channels, np.uint8, (width + 1) // 2, (height + 1) // 2)
    err = lib().ko_blur_and_downsample_u8(_ptr(src), _stride(src), width, height, _ptr(dst), _stride(dst),
                                          channels, border, int(ext), int(border_value), nthreads)
    return err, dst


def sobel_3x3_s16_u8(src, width, height, channels, horizontal, *, nthreads=1, dst=None):
    """Sobel x (horizontal=True) or y derivative of a u8 image as s16
    (kleidicv/src/filters/sobel_api.cpp:22-76, sobel_neon.cpp)."""
    if dst is None and src is not None:
        dst = _out_like(src, width, height, channels, np.int16)
    fn = lib().ko_sobel_3x3_horizontal_s16_u8 if horizontal else lib().ko_sobel_3x3_vertical_s16_u8
    err = fn(_ptr(src), _stride(src), _ptr(dst), _stride(dst), width, height, channels, nthreads)
    return err, dst


# --- median blur (kleidicv/src/filters/median_blur_api.cpp, filters/median_blur.h:148-193)

MEDIAN_DTYPES = {"s8": np.int8, "u8": np.uint8, "u16": np.uint16, "s16": np.int16, "u32": np.uint32,
                 "s32": np.int32, "f32": np.float32}


def median_blur_check(dtype, src_null, src_stride, dst_null, dst_stride, width, height, channels, kw, kh,
                      border, same_buffer=False):
    """Error code of kleidicv_median_blur_<dtype>, in the reference's order:
    pointers and strides, image size, then the NOT_IMPLEMENTED conditions."""
    es = np.dtype(MEDIAN_DTYPES[dtype]).itemsize
    if src_null:
        return NULL_POINTER
    if height > 1 and src_stride % es:
        return ALIGNMENT
    if dst_null:
        return NULL_POINTER
    if height > 1 and dst_stride % es:
        return ALIGNMENT
    if width * height > (1 << 48) - 1:
        return RANGE
    kmax = 255 if dtype == "u8" else 7
    ok = (not same_buffer and channels <= 4 and height >= kh - 1 and width >= kw - 1 and kw == kh
          and 3 <= kw <= kmax and kw % 2 == 1 and border in (1, 2, 3, 4))
    return OK if ok else NOT_IMPLEMENTED


def median_blur(src, width, height, channels, ksize, border, out_rows=None):
    """The reference test's model (test/api/test_median_blur.cpp:108-186): for
    every element, sort the border-mapped K x K window (same channel) and take
    the middle value.  `src` is 2-D (rows x elements, any padding).  With
    `out_rows` only those destination rows are computed (in that order)."""
    r = ksize // 2
    rows = np.array([border_map(i, height, border) for i in range(-r, height + r)])
    cols = np.array([border_map(i, width, border) for i in range(-r, width + r)])
    img = np.asarray(src)[:height, : width * channels].reshape(height, width, channels)
    padded = img[rows][:, cols]  # (h + 2r, w + 2r, c)
    mid = (ksize * ksize) // 2
    want = list(range(height)) if out_rows is None else list(out_rows)
    out = np.empty((len(want), width, channels), img.dtype)
    # Rows in chunks of at most ~32 M window elements.
    step = max(1, (32 << 20) // max(1, width * channels * ksize * ksize))
    for i in range(0, len(want), step):
        chunk = want[i:i + step]
        win = np.stack([np.lib.stride_tricks.sliding_window_view(padded[y:y + ksize], (ksize, ksize),
                                                                 axis=(0, 1))[0] for y in chunk])
        flat = win.reshape(len(chunk), width, channels, ksize * ksize)
        out[i:i + len(chunk)] = np.partition(flat, mid, axis=-1)[..., mid]
    return out.reshape(len(want), width * channels)


# --- LK optical-flow pyramid (kleidicv/include/kleidicv/analysis/build_optical_flow_pyr_lk_pyramid.h)

MAX_LK_WINDOW = 2047  # KLEIDICV_MAX_OPTICAL_FLOW_PYR_LK_WINDOW_SIZE, kleidicv.h:119


def lk_level_count(src_stride, width, height, channels, level_count, window_w, window_h):
    """validate_and_compute_build_optical_flow_pyr_lk_levels (:18-58): (error, levels)."""
    if (width == 0 or height == 0 or channels == 0 or channels > 4 or level_count == 0 or window_w <= 2
            or window_h <= 2 or window_w > MAX_LK_WINDOW or window_h > MAX_LK_WINDOW):
        return RANGE, 0
    if height > 1 and src_stride < width * channels:
        return RANGE, 0
    n, w, h = 0, width, height
    for _ in range(level_count):
        n += 1
        nw, nh = (w + 1) // 2, (h + 1) // 2
        if nw <= window_w or nh <= window_h:
            break
        w, h = nw, nh
    return OK, n


def reflect_101_index(i, n):
    """border_index_reflect_101 (:471-485): folds until inside [0, n)."""
    if n <= 1:
        return 0
    while i < 0 or i >= n:
        i = -i if i < 0 else 2 * n - i - 2
    return i


def lk_pyramid(src, width, height, channels, level_count, window_w, window_h):
    """The pyramid of create() (:306-383): per level the image with a
    reflect-101 border of (window_w, window_h) pixels and the interleaved
    (dx, dy) Scharr derivatives (s16, width x height x 2C) computed from the
    reflect-101 1-pixel ring.  Returns (error, [level dicts])."""
    err, n = lk_level_count(src.strides[0] if src.ndim == 2 else width * channels, width, height, channels,
                            level_count, window_w, window_h)
    if err != OK:
        return err, []
    bw, bh = window_w, window_h
    levels = []
    img = np.ascontiguousarray(src[:height, : width * channels])
    w, h = width, height
    for lvl in range(n):
        if lvl > 0:
            e, img = blur_and_downsample_u8(img, w, h, channels, REVERSE)
            assert e == OK
            w, h = (w + 1) // 2, (h + 1) // 2
        ys = np.array([reflect_101_index(y, h) for y in range(-bh, h + bh)])
        xs = np.array([reflect_101_index(x, w) for x in range(-bw, w + bw)])
        px = img.reshape(h, w, channels)
        bordered = px[ys][:, xs].reshape(h + 2 * bh, (w + 2 * bw) * channels)
        ring = px[[reflect_101_index(y, h) for y in range(-1, h + 1)]][:, [reflect_101_index(x, w) for x in range(-1, w + 1)]]
        ring = ring.astype(np.int32)
        dx = (3 * (ring[:-2, 2:] - ring[:-2, :-2]) + 10 * (ring[1:-1, 2:] - ring[1:-1, :-2]) +
              3 * (ring[2:, 2:] - ring[2:, :-2]))
        dy = (3 * (ring[2:, :-2] - ring[:-2, :-2]) + 10 * (ring[2:, 1:-1] - ring[:-2, 1:-1]) +
              3 * (ring[2:, 2:] - ring[:-2, 2:]))
        scharr = np.stack([dx, dy], axis=-1).astype(np.int16).reshape(h, w * channels * 2)
        levels.append(dict(width=w, height=h, image=bordered, scharr=scharr))
    return OK, levels


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print(LIB_PATH)
