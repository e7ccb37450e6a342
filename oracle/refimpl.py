"""ctypes front-end of the reference itself (KleidiCV + kleidicv_thread), built
natively on an AArch64 host by ``make -C oracle refnative`` into
``oracle/_ref/libkleidicv_ref.so``.

TEST INFRASTRUCTURE ONLY: the product library never imports this module.  It
serves the tests (as the bit-exact checker that pins the GPU path and the C
restatement in ``kcv_oracle.c`` to the reference's own output) and ``bench.py``
(the reference CPU path, ``kleidicv_thread_*`` on all host cores, timed as the
CPU baseline and the reference arm).

The library only exists where it can be built: an AArch64 host with the path's
reference sources staged in ``oracle/_ref/src`` (``make -C oracle ref`` stages
them from a reference tree).  ``status()`` says why it is missing otherwise.

Images are 2-D numpy arrays whose first axis is the row; row strides are
``array.strides[0]``, as in ``oracle.py``.
"""
from __future__ import annotations

import ctypes
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
LIB_PATH = os.path.join(REF_DIR, "libkleidicv_ref.so")
SRC_MARK = os.path.join(REF_DIR, "src", "kleidicv", "include", "kleidicv", "kleidicv.h")
LOG_PATH = os.path.join(REF_DIR, "refnative.log")

OK = 0
_lib = None
_status = None


def staged() -> bool:
    return os.path.exists(SRC_MARK)


def native_host() -> bool:
    return platform.machine() in ("aarch64", "arm64")


def build(jobs: int | None = None) -> str | None:
    """Builds the reference library when this host can (AArch64, sources staged).
    Returns None on success, else a one-line reason.  The full compiler output
    of a failed build is kept in oracle/_ref/refnative.log."""
    if not native_host():
        return f"host is {platform.machine()}, the reference is AArch64-only"
    if not staged():
        return "reference sources are not staged in oracle/_ref/src"
    jobs = jobs or os.cpu_count() or 4
    r = subprocess.run(["make", "-s", f"-j{jobs}", "-C", HERE, "refnative"], capture_output=True, text=True)
    with open(LOG_PATH, "w") as f:
        f.write(r.stdout + r.stderr)
    if r.returncode != 0:
        tail = (r.stdout + r.stderr).strip().splitlines()[-1:] or ["?"]
        return f"reference build failed: {tail[0][:200]}"
    return None


def status() -> str | None:
    """None when the reference library is loadable, else why it is not."""
    global _status
    if _lib is not None:
        return None
    if _status is None:
        try:
            lib()
        except OSError as e:
            _status = str(e)
    return _status


def available() -> bool:
    return status() is None


def lib():
    global _lib, _status
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        why = build()
        if why is not None:
            _status = why
            raise OSError(why)
    L = ctypes.CDLL(LIB_PATH)
    sz, vp, f, i, u = ctypes.c_size_t, ctypes.c_void_p, ctypes.c_float, ctypes.c_int, ctypes.c_uint
    L.ref_pool_create.argtypes = [u]
    L.ref_pool_create.restype = vp
    L.ref_pool_destroy.argtypes = [vp]
    L.ref_pool_destroy.restype = None
    L.ref_gaussian_blur_u8.argtypes = [vp, sz, vp, sz, sz, sz, sz, sz, sz, f, f, i]
    L.ref_thread_gaussian_blur_u8.argtypes = [vp] + L.ref_gaussian_blur_u8.argtypes
    for n in ("u8", "u16"):
        getattr(L, f"ref_separable_filter_2d_{n}").argtypes = [vp, sz, vp, sz, sz, sz, sz, vp, sz, vp, sz, i]
        getattr(L, f"ref_thread_separable_filter_2d_{n}").argtypes = [vp, vp, sz, vp, sz, sz, sz, sz, vp, sz, vp, sz,
                                                                       i]
    L.ref_blur_and_downsample_u8.argtypes = [vp, sz, sz, sz, vp, sz, sz, i]
    L.ref_thread_blur_and_downsample_u8.argtypes = [vp] + L.ref_blur_and_downsample_u8.argtypes
    for n in ("horizontal", "vertical"):
        getattr(L, f"ref_sobel_3x3_{n}_s16_u8").argtypes = [vp, sz, vp, sz, sz, sz, sz]
    L.ref_thread_sobel_3x3_horizontal_s16_u8.argtypes = [vp, vp, sz, vp, sz, sz, sz, sz]
    for n in ("s8", "u8", "u16", "s16", "u32", "s32", "f32"):
        getattr(L, f"ref_median_blur_{n}").argtypes = [vp, sz, vp, sz, sz, sz, sz, sz, sz, i]
    L.ref_thread_median_blur_u8.argtypes = [vp, vp, sz, vp, sz, sz, sz, sz, sz, sz, i]
    L.ref_lk_pyramid_build.argtypes = [ctypes.POINTER(vp), vp, sz, sz, sz, sz, sz, sz, sz]
    L.ref_lk_pyramid_level_count.argtypes = [vp, ctypes.POINTER(sz)]
    for n in ("image", "scharr"):
        getattr(L, f"ref_lk_pyramid_{n}_level").argtypes = [vp, sz, ctypes.POINTER(vp), ctypes.POINTER(sz),
                                                            ctypes.POINTER(sz), ctypes.POINTER(sz)]
    L.ref_lk_pyramid_release.argtypes = [vp]
    L.ref_sve_vector_bytes.argtypes = []
    _lib = L
    return L


def _ptr(a):
    return None if a is None else a.ctypes.data


def _stride(a):
    return 0 if a is None else int(a.strides[0])


def _out(rows, row_elems, dtype):
    return np.zeros((max(rows, 1), max(row_elems, 1)), dtype)


_MEDIAN = {np.dtype(np.int8): "s8", np.dtype(np.uint8): "u8", np.dtype(np.uint16): "u16",
           np.dtype(np.int16): "s16", np.dtype(np.uint32): "u32", np.dtype(np.int32): "s32",
           np.dtype(np.float32): "f32"}


class Pool:
    """A persistent worker pool (``threads`` workers including the caller) that
    drives the reference's ``kleidicv_thread_*`` entry points."""

    def __init__(self, threads: int):
        self.threads = int(threads)
        self.handle = lib().ref_pool_create(self.threads)

    def close(self):
        if self.handle:
            lib().ref_pool_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def gaussian_blur_u8(src, width, height, channels, ksize, sigma, border, *, dst=None, ksize_y=None,
                     sigma_y=None, pool: Pool | None = None):
    if dst is None and src is not None:
        dst = _out(height, width * channels, np.uint8)
    args = (_ptr(src), _stride(src), _ptr(dst), _stride(dst), width, height, channels, ksize,
            ksize if ksize_y is None else ksize_y, float(sigma), float(sigma if sigma_y is None else sigma_y),
            border)
    err = lib().ref_thread_gaussian_blur_u8(pool.handle, *args) if pool else lib().ref_gaussian_blur_u8(*args)
    return err, dst


def separable_filter_2d(src, width, height, channels, kernel_x, kernel_y, border, *, dst=None,
                        pool: Pool | None = None):
    dtype = np.dtype(src.dtype)
    name = {np.dtype(np.uint8): "u8", np.dtype(np.uint16): "u16"}[dtype]
    if dst is None:
        dst = _out(height, width * channels, dtype)
    kx = np.ascontiguousarray(kernel_x, dtype)
    ky = np.ascontiguousarray(kernel_y, dtype)
    args = (_ptr(src), _stride(src), _ptr(dst), _stride(dst), width, height, channels, kx.ctypes.data, len(kx),
            ky.ctypes.data, len(ky), border)
    if pool:
        err = getattr(lib(), f"ref_thread_separable_filter_2d_{name}")(pool.handle, *args)
    else:
        err = getattr(lib(), f"ref_separable_filter_2d_{name}")(*args)
    return err, dst


def blur_and_downsample_u8(src, width, height, channels, border, *, dst=None, pool: Pool | None = None):
    if dst is None:
        dst = _out((height + 1) // 2, (width + 1) // 2 * channels, np.uint8)
    args = (_ptr(src), _stride(src), width, height, _ptr(dst), _stride(dst), channels, border)
    err = lib().ref_thread_blur_and_downsample_u8(pool.handle, *args) if pool else \
        lib().ref_blur_and_downsample_u8(*args)
    return err, dst


def sobel_3x3_s16_u8(src, width, height, channels, horizontal, *, dst=None):
    if dst is None:
        dst = _out(height, width * channels, np.int16)
    fn = lib().ref_sobel_3x3_horizontal_s16_u8 if horizontal else lib().ref_sobel_3x3_vertical_s16_u8
    err = fn(_ptr(src), _stride(src), _ptr(dst), _stride(dst), width, height, channels)
    return err, dst


def median_blur(src, width, height, channels, ksize, border, *, dst=None):
    dtype = np.dtype(src.dtype)
    if dst is None:
        dst = _out(height, width * channels, dtype)
    err = getattr(lib(), f"ref_median_blur_{_MEDIAN[dtype]}")(_ptr(src), _stride(src), _ptr(dst), _stride(dst),
                                                              width, height, channels, ksize, ksize, border)
    return err, dst


def lk_pyramid(src, width, height, channels, levels, window_w, window_h):
    """Builds the reference LK pyramid and copies every level out.
    Returns (err, [(image, scharr), ...]) with image rows of width*channels u8
    and scharr rows of width*channels*2 s16 (interleaved dx, dy)."""
    L = lib()
    handle = ctypes.c_void_p()
    err = L.ref_lk_pyramid_build(ctypes.byref(handle), _ptr(src), _stride(src), width, height, channels, levels,
                                 window_w, window_h)
    if err != OK:
        return err, []
    try:
        count = ctypes.c_size_t()
        assert L.ref_lk_pyramid_level_count(handle, ctypes.byref(count)) == OK
        out = []
        for lv in range(count.value):
            p, s, w, h = ctypes.c_void_p(), ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t()
            assert L.ref_lk_pyramid_image_level(handle, lv, ctypes.byref(p), ctypes.byref(s), ctypes.byref(w),
                                                ctypes.byref(h)) == OK
            img = _copy_rows(p.value, h.value, w.value * channels, s.value, np.uint8)
            assert L.ref_lk_pyramid_scharr_level(handle, lv, ctypes.byref(p), ctypes.byref(s), ctypes.byref(w),
                                                 ctypes.byref(h)) == OK
            sch = _copy_rows(p.value, h.value, w.value * channels * 2, s.value, np.int16)
            out.append((img, sch))
        return OK, out
    finally:
        L.ref_lk_pyramid_release(handle)


def _copy_rows(ptr, rows, row_elems, stride, dtype):
    es = np.dtype(dtype).itemsize
    raw = (ctypes.c_uint8 * (stride * (rows - 1) + row_elems * es)).from_address(ptr)
    flat = np.frombuffer(raw, np.uint8)
    return np.stack([flat[r * stride: r * stride + row_elems * es].view(dtype) for r in range(rows)]).copy()


def host_info() -> dict:
    """CPU model, logical core count and SVE vector length of this host."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    feats = set()
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("features", "flags")):
                    feats = set(line.split(":", 1)[1].split())
                    break
    except OSError:
        pass
    isa = [n for n, f in (("NEON", "asimd"), ("SVE", "sve"), ("SVE2", "sve2"), ("SME", "sme")) if f in feats]
    info = {"cpu_model": model, "cores": os.cpu_count(), "arch": platform.machine(),
            "isa": "+".join(isa) or None,
            # The reference picks its SVE2 code paths only when the kernel reports SVE2
            # (AT_HWCAP2); otherwise every function runs its NEON path.
            "reference_backend": "SVE2 where the reference selects it, else NEON" if "sve2" in feats else "NEON"}
    if available():
        vb = int(lib().ref_sve_vector_bytes())
        info["sve_vector_bits"] = vb * 8 if vb else None
    return info
