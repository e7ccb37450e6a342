"""Python binding of the GB300 separable-filter library (libkleidicv_gpu.so).

The product is the C ABI declared in include/kleidicv_gpu.h; this module binds
it with ctypes so that Python callers (the tests, the benchmark, a serving
front-end) can drive it with raw device pointers or with torch CUDA tensors.
Function names, argument order and error codes are those of KleidiCV's C API
(kleidicv/include/kleidicv/kleidicv.h:2091-2218) plus the trailing context.

There is no CPU fallback: if the shared library is missing, or no sm_103
device is present, the calls fail loudly.
"""
from __future__ import annotations

import ctypes
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libkleidicv_gpu.so")

# kleidicv_error_t (kleidicv/include/kleidicv/ctypes.h:26-41) + GPU extensions
OK, NOT_IMPLEMENTED, NULL_POINTER, RANGE, ALLOCATION, ALIGNMENT, CONTEXT_MISMATCH = range(7)
ERROR_CUDA, ERROR_NO_DEVICE, ERROR_TIMEOUT, ERROR_BUSY, ERROR_NOT_READY = 0x100, 0x101, 0x102, 0x103, 0x104
# kleidicv_border_type_t (ctypes.h:60-79)
CONSTANT, REPLICATE, REFLECT, WRAP, REVERSE, TRANSPARENT, NONE = range(7)
# kleidicv_gpu_op_t
OP_GAUSSIAN_BLUR_U8, OP_SEPARABLE_U8, OP_SEPARABLE_U16, OP_SEPARABLE_S16, OP_BLUR_AND_DOWNSAMPLE_U8 = range(5)

ERROR_NAMES = {0: "OK", 1: "NOT_IMPLEMENTED", 2: "NULL_POINTER", 3: "RANGE", 4: "ALLOCATION",
               5: "ALIGNMENT", 6: "CONTEXT_MISMATCH", 0x100: "CUDA", 0x101: "NO_DEVICE",
               0x102: "TIMEOUT", 0x103: "BUSY", 0x104: "NOT_READY"}

_sz, _vp, _f, _i, _u8, _u16, _i16 = (ctypes.c_size_t, ctypes.c_void_p, ctypes.c_float, ctypes.c_int,
                                     ctypes.c_uint8, ctypes.c_uint16, ctypes.c_int16)


class Request(ctypes.Structure):
    """kleidicv_gpu_request_t"""
    _fields_ = [("op", _i), ("src", _vp), ("src_stride", _sz), ("dst", _vp), ("dst_stride", _sz),
                ("width", _sz), ("height", _sz), ("channels", _sz), ("kernel_width", _sz),
                ("kernel_height", _sz), ("sigma_x", _f), ("sigma_y", _f),
                ("kernel_x", ctypes.c_int32 * 5), ("kernel_y", ctypes.c_int32 * 5),
                ("border_type", _i), ("border_value", ctypes.c_int32),
                ("allow_extensions", ctypes.c_int32)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("pool_limit_bytes", _sz), ("max_inflight_batches", _i), ("max_batch_requests", _i),
                ("max_queue", _i), ("max_batch_bytes", _sz)]


class Pyramid(ctypes.Structure):
    """kleidicv_gpu_pyramid_t: one image pyramid of a kleidicv_gpu_build_pyramids_u8 call."""
    _fields_ = [("src", _vp), ("src_stride", _sz), ("src_width", _sz), ("src_height", _sz), ("channels", _sz),
                ("levels", _sz), ("dst", _vp), ("dst_strides", _vp), ("border_type", _i)]


class ThreadMT(ctypes.Structure):
    """kleidicv_thread_multithreading: the caller's scheduler (function pointer) and its data."""
    _fields_ = [("parallel", _vp), ("parallel_data", _vp)]


class Completion(ctypes.Structure):
    _fields_ = [("id", ctypes.c_uint64), ("status", _i), ("arrival_s", ctypes.c_double),
                ("admitted_s", ctypes.c_double), ("completed_s", ctypes.c_double)]


# name -> (restype, argtypes).  This table is also the list of exported symbols
# the CPU tests check against include/kleidicv_gpu.h.
SIGNATURES = {
    "kleidicv_gpu_context_create": (_i, [ctypes.POINTER(_vp), _i, _vp, _sz]),
    "kleidicv_gpu_context_destroy": (_i, [_vp]),
    "kleidicv_gpu_context_set_stream": (_i, [_vp, _vp]),
    "kleidicv_gpu_context_get_stream": (_vp, [_vp]),
    "kleidicv_gpu_context_synchronize": (_i, [_vp]),
    "kleidicv_gpu_context_fail_next_allocations": (None, [_vp, _i]),
    "kleidicv_gpu_context_launch_count": (ctypes.c_uint64, [_vp]),
    "kleidicv_gpu_context_set_tile_shape": (_i, [_vp, _i, _i, _i, _i]),
    "kleidicv_gpu_gaussian_blur_u8": (_i, [_vp, _sz, _vp, _sz, _sz, _sz, _sz, _sz, _sz, _f, _f, _i, _vp]),
    "kleidicv_gpu_gaussian_blur_u8_ex": (_i, [_vp, _sz, _vp, _sz, _sz, _sz, _sz, _sz, _sz, _f, _f, _i,
                                              _u8, _vp]),
    "kleidicv_gpu_separable_filter_2d_u8": (_i, [_vp, _sz, _vp, _sz, _sz, _sz, _sz, _vp, _sz, _vp, _sz,
                                                 _i, _vp]),
    "kleidicv_gpu_separable_filter_2d_u16": (_i, [_vp, _sz, _vp, _sz, _sz, _sz, _sz, _vp, _sz, _vp, _sz,
                                                  _i, _vp]),
    "kleidicv_gpu_separable_filter_2d_u8_ex": (_i, [_vp, _sz, _vp, _sz, _sz, _sz, _sz, _vp, _sz, _vp,
                                                    _sz, _i, _u8, _vp]),
    "kleidicv_gpu_separable_filter_2d_u16_ex": (_i, [_vp, _sz, _vp, _sz, _sz, _sz, _sz, _vp, _sz, _vp,
                                                     _sz, _i, _u16, _vp]),
    "kleidicv_gpu_separable_filter_2d_s16_ex": (_i, [_vp, _sz, _vp, _sz, _sz, _sz, _sz, _vp, _sz, _vp,
                                                     _sz, _i, _i16, _vp]),
    "kleidicv_gpu_blur_and_downsample_u8": (_i, [_vp, _sz, _sz, _sz, _vp, _sz, _sz, _i, _vp]),
    "kleidicv_gpu_blur_and_downsample_u8_ex": (_i, [_vp, _sz, _sz, _sz, _vp, _sz, _sz, _i, _u8, _vp]),
    "kleidicv_gpu_sobel_3x3_horizontal_s16_u8": (_i, [_vp, _sz, _vp, _sz, _sz, _sz, _sz, _vp]),
    "kleidicv_gpu_sobel_3x3_vertical_s16_u8": (_i, [_vp, _sz, _vp, _sz, _sz, _sz, _sz, _vp]),
    **{f"kleidicv_gpu_median_blur_{t}": (_i, [_vp, _sz, _vp, _sz, _sz, _sz, _sz, _sz, _sz, _i, _vp])
       for t in ("s8", "u8", "u16", "s16", "u32", "s32", "f32")},
    # Threaded API (include/kleidicv_gpu_thread.h): host images, the caller's scheduler.
    "kleidicv_gpu_thread_gaussian_blur_u8": (_i, [_vp, _sz, _vp, _sz, _sz, _sz, _sz, _sz, _sz, _f, _f, _i,
                                                  ThreadMT]),
    "kleidicv_gpu_thread_separable_filter_2d_u8": (_i, [_vp, _sz, _vp, _sz, _sz, _sz, _sz, _vp, _sz, _vp, _sz,
                                                        _i, ThreadMT]),
    "kleidicv_gpu_thread_separable_filter_2d_u16": (_i, [_vp, _sz, _vp, _sz, _sz, _sz, _sz, _vp, _sz, _vp, _sz,
                                                         _i, ThreadMT]),
    "kleidicv_gpu_thread_blur_and_downsample_u8": (_i, [_vp, _sz, _sz, _sz, _vp, _sz, _sz, _i, ThreadMT]),
    "kleidicv_gpu_thread_sobel_3x3_horizontal_s16_u8": (_i, [_vp, _sz, _vp, _sz, _sz, _sz, _sz, ThreadMT]),
    "kleidicv_gpu_thread_sobel_3x3_vertical_s16_u8": (_i, [_vp, _sz, _vp, _sz, _sz, _sz, _sz, ThreadMT]),
    **{f"kleidicv_gpu_thread_median_blur_{t}": (_i, [_vp, _sz, _vp, _sz, _sz, _sz, _sz, _sz, _sz, _i, ThreadMT])
       for t in ("s8", "u8", "u16", "s16", "u32", "s32", "f32")},
    # Asynchronous threaded calls: ..., mt, done callback, user data, handle out.
    "kleidicv_gpu_thread_gaussian_blur_u8_async": (_i, [_vp, _sz, _vp, _sz, _sz, _sz, _sz, _sz, _sz, _f, _f,
                                                        _i, ThreadMT, _vp, _vp, ctypes.POINTER(_vp)]),
    "kleidicv_gpu_thread_separable_filter_2d_u8_async": (_i, [_vp, _sz, _vp, _sz, _sz, _sz, _sz, _vp, _sz, _vp,
                                                              _sz, _i, ThreadMT, _vp, _vp, ctypes.POINTER(_vp)]),
    "kleidicv_gpu_thread_separable_filter_2d_u16_async": (_i, [_vp, _sz, _vp, _sz, _sz, _sz, _sz, _vp, _sz, _vp,
                                                               _sz, _i, ThreadMT, _vp, _vp, ctypes.POINTER(_vp)]),
    "kleidicv_gpu_thread_blur_and_downsample_u8_async": (_i, [_vp, _sz, _sz, _sz, _vp, _sz, _sz, _i, ThreadMT,
                                                              _vp, _vp, ctypes.POINTER(_vp)]),
    "kleidicv_gpu_async_query": (_i, [_vp]),
    "kleidicv_gpu_async_wait": (_i, [_vp]),
    "kleidicv_gpu_async_release": (_i, [_vp]),
    "kleidicv_gpu_thread_pool_create": (_i, [ctypes.POINTER(_vp), ctypes.c_uint]),
    "kleidicv_gpu_thread_pool_destroy": (_i, [_vp]),
    "kleidicv_gpu_thread_pool_parallel": (_i, [_vp, _vp, _vp, ctypes.c_uint]),
    # OpenCV custom-HAL shim (include/kleidicv_gpu_hal.h): OpenCV's hook signatures.
    "kleidicv_gpu_hal_separable_filter_2d": (_i, [_vp, _sz, _i, _vp, _sz, _i, _i, _i, _i, _i, _i, _i, _vp, _i,
                                                  _vp, _i, _i, _i, _i, ctypes.c_double, _i]),
    "kleidicv_gpu_hal_gaussian_blur_binomial": (_i, [_vp, _sz, _vp, _sz, _i, _i, _i, _i, _sz, _sz, _sz, _sz,
                                                     _sz, _i]),
    "kleidicv_gpu_hal_gaussian_blur": (_i, [_vp, _sz, _vp, _sz, _i, _i, _i, _i, _sz, _sz, _sz, _sz, _sz, _sz,
                                            ctypes.c_double, ctypes.c_double, _i]),
    "kleidicv_gpu_hal_pyrdown": (_i, [_vp, _sz, _i, _i, _vp, _sz, _i, _i, _i, _i, _i]),
    "kleidicv_gpu_hal_sobel": (_i, [_vp, _sz, _vp, _sz, _i, _i, _i, _i, _i, _i, _i, _i, _i, _i, _i, _i,
                                    ctypes.c_double, ctypes.c_double, _i]),
    "kleidicv_gpu_build_pyramid_u8": (_i, [_vp, _sz, _sz, _sz, _sz, _sz, _vp, _vp, _i, _vp]),
    "kleidicv_gpu_build_pyramids_u8": (_i, [ctypes.POINTER(Pyramid), _sz, ctypes.POINTER(_i), _vp]),
    "kleidicv_gpu_batch_plan_create": (_i, [ctypes.POINTER(Request), _sz, ctypes.POINTER(_i),
                                            ctypes.POINTER(_vp), _vp]),
    "kleidicv_gpu_batch_plan_launch": (_i, [_vp, _i, _vp]),
    "kleidicv_gpu_batch_plan_destroy": (_i, [_vp]),
    "kleidicv_gpu_batch_plan_tile_count": (_sz, [_vp]),
    "kleidicv_gpu_batch_submit": (_i, [ctypes.POINTER(Request), _sz, ctypes.POINTER(_i), _vp]),
    "kleidicv_gpu_server_create": (_i, [ctypes.POINTER(ServerConfig), _i, ctypes.POINTER(_vp)]),
    "kleidicv_gpu_server_destroy": (_i, [_vp]),
    "kleidicv_gpu_server_alloc": (_vp, [_vp, _sz]),
    "kleidicv_gpu_server_free": (None, [_vp, _vp]),
    "kleidicv_gpu_server_submit": (_i, [_vp, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_uint64)]),
    "kleidicv_gpu_server_poll": (_sz, [_vp, ctypes.POINTER(Completion), _sz, _i]),
    "kleidicv_gpu_server_now": (ctypes.c_double, [_vp]),
    "kleidicv_gpu_server_drain": (_i, [_vp]),
    "kleidicv_gpu_gaussian_half_kernel": (_i, [_sz, _f, ctypes.POINTER(_u8)]),
    "kleidicv_gpu_selftest_bounded_wait": (_i, [_vp, ctypes.c_uint64]),
    "kleidicv_gpu_build_optical_flow_pyr_lk_pyramid": (_i, [ctypes.POINTER(_vp), _vp, _sz, _sz, _sz, _sz, _sz,
                                                            _sz, _sz, _vp]),
    "kleidicv_gpu_optical_flow_pyr_lk_pyramid_release": (_i, [_vp]),
    "kleidicv_gpu_lk_pyramid_level_count": (_sz, [_vp]),
    "kleidicv_gpu_lk_pyramid_level": (_i, [_vp, _sz, ctypes.POINTER(_sz), ctypes.POINTER(_sz),
                                           ctypes.POINTER(_vp), ctypes.POINTER(_sz), ctypes.POINTER(_vp),
                                           ctypes.POINTER(_sz), ctypes.POINTER(_sz), ctypes.POINTER(_sz)]),
    "kleidicv_gpu_gaussian_blur_u8_noalloc": (_i, [_vp, _sz, _vp, _sz, _sz, _sz, _sz, _sz, _sz, _f, _f,
                                                   _i, _vp]),
}
# The `_sme` twins take the argument lists of their base entries.
SME_TWINS = ("kleidicv_gpu_gaussian_blur_u8", "kleidicv_gpu_separable_filter_2d_u8",
             "kleidicv_gpu_separable_filter_2d_u16", "kleidicv_gpu_blur_and_downsample_u8",
             "kleidicv_gpu_sobel_3x3_horizontal_s16_u8", "kleidicv_gpu_sobel_3x3_vertical_s16_u8")
for _name in SME_TWINS:
    SIGNATURES[_name + "_sme"] = SIGNATURES[_name]

_lib = None


def lib(path: str | None = None) -> ctypes.CDLL:
    """Loads libkleidicv_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise RuntimeError(f"{p} is missing: run build() first (there is no CPU fallback)")
        l = ctypes.CDLL(p)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(l, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _lib = l
    return _lib


def build(force: bool = False) -> str:
    from importlib import util

    spec = util.spec_from_file_location("_kcv_build", os.path.join(HERE, "build.py"))
    mod = util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force)


def half_kernel(ksize: int, sigma: float):
    out = (ctypes.c_uint8 * 128)()
    ok = lib().kleidicv_gpu_gaussian_half_kernel(ksize, sigma, out)
    return [int(v) for v in out[: ksize // 2 + 1]] if ok else None


class Context:
    """kleidicv_gpu_context_t bound to a device and a CUDA stream handle."""

    def __init__(self, device: int = 0, stream: int | None = None, pool_limit: int = 0):
        h = ctypes.c_void_p()
        err = lib().kleidicv_gpu_context_create(ctypes.byref(h), device, stream or None, pool_limit)
        if err != OK:
            raise RuntimeError(f"kleidicv_gpu_context_create failed: {ERROR_NAMES.get(err, err)}")
        self.handle = h

    @classmethod
    def for_torch(cls, device: int = 0, pool_limit: int = 0):
        """Context on torch's current stream of `device`."""
        import torch

        return cls(device, torch.cuda.current_stream(device).cuda_stream, pool_limit)

    def set_stream(self, stream: int | None):
        lib().kleidicv_gpu_context_set_stream(self.handle, stream or None)

    def synchronize(self) -> int:
        return lib().kleidicv_gpu_context_synchronize(self.handle)

    def launch_count(self) -> int:
        return lib().kleidicv_gpu_context_launch_count(self.handle)

    def set_tile_shape(self, threads=0, tile_rows=0, stage_rows=4, stages=4) -> int:
        return lib().kleidicv_gpu_context_set_tile_shape(self.handle, threads, tile_rows, stage_rows, stages)

    def fail_next_allocations(self, n: int):
        lib().kleidicv_gpu_context_fail_next_allocations(self.handle, n)

    def close(self):
        if self.handle:
            lib().kleidicv_gpu_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        # At interpreter exit the CUDA runtime may already be gone: leave the
        # release to process teardown instead of calling into it.
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


def _h(ctx):
    return None if ctx is None else ctx.handle


def _k(vals, ctype):
    if vals is None:
        return None
    arr = (ctype * len(vals))(*[int(v) for v in vals])
    return ctypes.cast(arr, ctypes.c_void_p), arr


# --- C-API mirrors (raw pointers and byte strides) -------------------------

def gaussian_blur_u8(src, src_stride, dst, dst_stride, width, height, channels, kernel_width,
                     kernel_height, sigma_x, sigma_y, border_type, ctx=None, border_value=None):
    if border_value is None:
        return lib().kleidicv_gpu_gaussian_blur_u8(src, src_stride, dst, dst_stride, width, height,
                                                   channels, kernel_width, kernel_height, sigma_x,
                                                   sigma_y, border_type, _h(ctx))
    return lib().kleidicv_gpu_gaussian_blur_u8_ex(src, src_stride, dst, dst_stride, width, height,
                                                  channels, kernel_width, kernel_height, sigma_x,
                                                  sigma_y, border_type, border_value, _h(ctx))


def gaussian_blur_u8_noalloc(src, src_stride, dst, dst_stride, width, height, channels,
                             kernel_width, kernel_height, sigma_x, sigma_y, border_type, stream=None):
    """Allocation-free two-pass Gaussian on a raw cudaStream_t handle (no context)."""
    return lib().kleidicv_gpu_gaussian_blur_u8_noalloc(src, src_stride, dst, dst_stride, width, height,
                                                       channels, kernel_width, kernel_height, sigma_x,
                                                       sigma_y, border_type, stream or None)


def separable_filter_2d(dtype, src, src_stride, dst, dst_stride, width, height, channels, kernel_x,
                        kernel_width, kernel_y, kernel_height, border_type, ctx=None,
                        border_value=None):
    """dtype: 'u8' | 'u16' | 's16' (s16 exists only as an extension)."""
    ct = {"u8": ctypes.c_uint8, "u16": ctypes.c_uint16, "s16": ctypes.c_int16}[dtype]
    kx = _k(kernel_x, ct)
    ky = _k(kernel_y, ct)
    kxp = kx[0] if kx else None
    kyp = ky[0] if ky else None
    L = lib()
    if dtype == "s16":
        return L.kleidicv_gpu_separable_filter_2d_s16_ex(src, src_stride, dst, dst_stride, width, height,
                                                         channels, kxp, kernel_width, kyp, kernel_height,
                                                         border_type, border_value or 0, _h(ctx))
    if border_value is None:
        fn = getattr(L, f"kleidicv_gpu_separable_filter_2d_{dtype}")
        return fn(src, src_stride, dst, dst_stride, width, height, channels, kxp, kernel_width, kyp,
                  kernel_height, border_type, _h(ctx))
    fn = getattr(L, f"kleidicv_gpu_separable_filter_2d_{dtype}_ex")
    return fn(src, src_stride, dst, dst_stride, width, height, channels, kxp, kernel_width, kyp,
              kernel_height, border_type, border_value, _h(ctx))


def blur_and_downsample_u8(src, src_stride, src_width, src_height, dst, dst_stride, channels,
                           border_type, ctx=None, border_value=None):
    if border_value is None:
        return lib().kleidicv_gpu_blur_and_downsample_u8(src, src_stride, src_width, src_height, dst,
                                                         dst_stride, channels, border_type, _h(ctx))
    return lib().kleidicv_gpu_blur_and_downsample_u8_ex(src, src_stride, src_width, src_height, dst,
                                                        dst_stride, channels, border_type,
                                                        border_value, _h(ctx))


MEDIAN_TYPES = {"s8": "int8", "u8": "uint8", "u16": "uint16", "s16": "int16", "u32": "uint32", "s32": "int32",
                "f32": "float32"}


def median_blur(dtype, src, src_stride, dst, dst_stride, width, height, channels, kernel_width, kernel_height,
                border_type, ctx=None):
    """kleidicv_median_blur_<dtype> (kleidicv/src/filters/median_blur_api.cpp:42-242);
    dtype in s8, u8, u16, s16, u32, s32, f32."""
    fn = getattr(lib(), f"kleidicv_gpu_median_blur_{dtype}")
    return fn(src, src_stride, dst, dst_stride, width, height, channels, kernel_width, kernel_height, border_type,
              _h(ctx))


THREAD_CALLBACK = ctypes.CFUNCTYPE(_i, ctypes.c_uint, ctypes.c_uint, _vp)
THREAD_PARALLEL = ctypes.CFUNCTYPE(_i, THREAD_CALLBACK, _vp, _vp, ctypes.c_uint)


class ThreadPool:
    """The library's worker pool implementing the kleidicv_thread_parallel
    contract; `mt` is the kleidicv_thread_multithreading value to pass."""

    def __init__(self, threads: int = 0):
        h = _vp()
        err = lib().kleidicv_gpu_thread_pool_create(ctypes.byref(h), threads)
        if err != OK:
            raise RuntimeError(f"kleidicv_gpu_thread_pool_create failed: {ERROR_NAMES.get(err, err)}")
        self.handle = h.value
        fn = ctypes.cast(lib().kleidicv_gpu_thread_pool_parallel, _vp).value
        self.mt = ThreadMT(fn, self.handle)

    def close(self):
        if self.handle:
            lib().kleidicv_gpu_thread_pool_destroy(self.handle)
            self.handle = None


ASYNC_CALLBACK = ctypes.CFUNCTYPE(None, _i, _vp)


def serial_scheduler():
    """A scheduler written in Python: runs every task range on the calling
    thread (the reference's serial fallback).  Keep the returned pair alive
    while it is in use."""

    @THREAD_PARALLEL
    def parallel(callback, callback_data, parallel_data, task_count):
        return callback(0, task_count, callback_data)

    return ThreadMT(ctypes.cast(parallel, _vp).value, None), parallel


def sobel_3x3_horizontal_s16_u8(src, src_stride, dst, dst_stride, width, height, channels, ctx=None):
    """kleidicv_sobel_3x3_horizontal_s16_u8 (kleidicv/src/filters/sobel_api.cpp:37-43)."""
    return lib().kleidicv_gpu_sobel_3x3_horizontal_s16_u8(src, src_stride, dst, dst_stride, width, height,
                                                          channels, _h(ctx))


def sobel_3x3_vertical_s16_u8(src, src_stride, dst, dst_stride, width, height, channels, ctx=None):
    """kleidicv_sobel_3x3_vertical_s16_u8 (kleidicv/src/filters/sobel_api.cpp:53-58)."""
    return lib().kleidicv_gpu_sobel_3x3_vertical_s16_u8(src, src_stride, dst, dst_stride, width, height,
                                                        channels, _h(ctx))


def build_pyramid_u8(src, src_stride, src_width, src_height, channels, dsts, dst_strides,
                     border_type, ctx=None):
    n = len(dsts)
    dp = (ctypes.c_void_p * max(n, 1))(*dsts)
    ds = (ctypes.c_size_t * max(n, 1))(*dst_strides)
    return lib().kleidicv_gpu_build_pyramid_u8(src, src_stride, src_width, src_height, channels, n,
                                               ctypes.cast(dp, ctypes.c_void_p),
                                               ctypes.cast(ds, ctypes.c_void_p), border_type, _h(ctx))


class PyramidBatch:
    """The arguments of one kleidicv_gpu_build_pyramids_u8 call, converted once:
    pyramids is a list of (src, src_stride, width, height, channels, dsts,
    dst_strides, border).  launch() makes the call (repeatable)."""

    def __init__(self, pyramids):
        self.n = len(pyramids)
        self.arr = (Pyramid * max(self.n, 1))()
        self._keep = []
        for i, (src, ss, w, h, c, dsts, dss, border) in enumerate(pyramids):
            dp = (ctypes.c_void_p * max(len(dsts), 1))(*dsts)
            ds = (ctypes.c_size_t * max(len(dss), 1))(*dss)
            self._keep += [dp, ds]
            self.arr[i] = Pyramid(src, ss, w, h, c, len(dsts), ctypes.cast(dp, _vp), ctypes.cast(ds, _vp),
                                  border)
        self.statuses = (_i * max(self.n, 1))()

    def launch(self, ctx=None):
        """Returns (error, statuses)."""
        err = lib().kleidicv_gpu_build_pyramids_u8(self.arr, self.n, self.statuses, _h(ctx))
        return err, list(self.statuses)[:self.n]


def build_pyramids_u8(pyramids, ctx=None):
    """pyramids: list of (src, src_stride, width, height, channels, dsts, dst_strides, border).
    Returns (error, statuses)."""
    return PyramidBatch(pyramids).launch(ctx)


# --- Lucas-Kanade pyramid ---------------------------------------------------

class LKPyramid:
    """kleidicv_gpu_lk_pyramid_t: per-level bordered images and Scharr pairs on the GPU."""

    def __init__(self, src, src_stride, width, height, channels, level_count, window_width, window_height,
                 ctx=None):
        h = ctypes.c_void_p()
        err = lib().kleidicv_gpu_build_optical_flow_pyr_lk_pyramid(ctypes.byref(h), src, src_stride, width, height,
                                                                   channels, level_count, window_width,
                                                                   window_height, _h(ctx))
        self.error = err
        self.handle = h if err == OK else None

    def level_count(self) -> int:
        return lib().kleidicv_gpu_lk_pyramid_level_count(self.handle)

    def level(self, i):
        """(width, height, image_ptr, image_stride, scharr_ptr, scharr_stride, border_w, border_h)."""
        vals = [_sz() for _ in range(2)]
        img, sch = _vp(), _vp()
        istr, sstr, bw, bh = _sz(), _sz(), _sz(), _sz()
        err = lib().kleidicv_gpu_lk_pyramid_level(self.handle, i, ctypes.byref(vals[0]), ctypes.byref(vals[1]),
                                                  ctypes.byref(img), ctypes.byref(istr), ctypes.byref(sch),
                                                  ctypes.byref(sstr), ctypes.byref(bw), ctypes.byref(bh))
        if err != OK:
            raise RuntimeError(f"kleidicv_gpu_lk_pyramid_level: {ERROR_NAMES.get(err, err)}")
        return (vals[0].value, vals[1].value, img.value, istr.value, sch.value, sstr.value, bw.value, bh.value)

    def close(self):
        if self.handle:
            lib().kleidicv_gpu_optical_flow_pyr_lk_pyramid_release(self.handle)
            self.handle = None

    def __del__(self):
        # At interpreter exit the CUDA runtime may already be gone: leave the
        # release to process teardown instead of calling into it.
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


# --- batched execution -----------------------------------------------------

def make_request(op, src, src_stride, dst, dst_stride, width, height, channels, kernel_width=0,
                 kernel_height=0, sigma_x=0.0, sigma_y=0.0, kernel_x=None, kernel_y=None,
                 border_type=REPLICATE, border_value=0, allow_extensions=False):
    """kleidicv_gpu_request_t for one filter call (device pointers, byte strides)."""
    r = Request()
    r.op, r.src, r.src_stride, r.dst, r.dst_stride = op, src, src_stride, dst, dst_stride
    r.width, r.height, r.channels = width, height, channels
    r.kernel_width, r.kernel_height, r.sigma_x, r.sigma_y = kernel_width, kernel_height, sigma_x, sigma_y
    for i, v in enumerate(kernel_x or [0] * 5):
        r.kernel_x[i] = int(v)
    for i, v in enumerate(kernel_y or [0] * 5):
        r.kernel_y[i] = int(v)
    r.border_type, r.border_value, r.allow_extensions = border_type, int(border_value), int(allow_extensions)
    return r


class BatchPlan:
    """kleidicv_gpu_batch_plan_t: validated requests, tile work-lists, optional CUDA graph."""

    def __init__(self, requests, ctx=None):
        n = len(requests)
        self._reqs = (Request * max(n, 1))(*requests)
        self._statuses = (_i * max(n, 1))()
        h = ctypes.c_void_p()
        err = lib().kleidicv_gpu_batch_plan_create(self._reqs, n, self._statuses, ctypes.byref(h), _h(ctx))
        if err != OK:
            raise RuntimeError(f"kleidicv_gpu_batch_plan_create failed: {ERROR_NAMES.get(err, err)}")
        self.handle = h
        self.statuses = [int(self._statuses[i]) for i in range(n)]
        self.ctx = ctx

    def tile_count(self) -> int:
        return lib().kleidicv_gpu_batch_plan_tile_count(self.handle)

    def launch(self, use_graph=True) -> int:
        return lib().kleidicv_gpu_batch_plan_launch(self.handle, int(use_graph), _h(self.ctx))

    def close(self):
        if self.handle:
            lib().kleidicv_gpu_batch_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        # At interpreter exit the CUDA runtime may already be gone: leave the
        # release to process teardown instead of calling into it.
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


def batch_submit(requests, ctx=None):
    """One-shot batch: returns (error, per-request statuses)."""
    n = len(requests)
    reqs = (Request * max(n, 1))(*requests)
    st = (_i * max(n, 1))()
    err = lib().kleidicv_gpu_batch_submit(reqs, n, st, _h(ctx))
    return err, [int(st[i]) for i in range(n)]


# --- serving loop ----------------------------------------------------------

class Server:
    """kleidicv_gpu_server_t: continuous batching over a capped device pool."""

    def __init__(self, device=0, pool_limit_bytes=0, max_inflight_batches=0, max_batch_requests=0,
                 max_queue=0, max_batch_bytes=0):
        cfg = ServerConfig(pool_limit_bytes, max_inflight_batches, max_batch_requests, max_queue, max_batch_bytes)
        h = ctypes.c_void_p()
        err = lib().kleidicv_gpu_server_create(ctypes.byref(cfg), device, ctypes.byref(h))
        if err != OK:
            raise RuntimeError(f"kleidicv_gpu_server_create failed: {ERROR_NAMES.get(err, err)}")
        self.handle = h

    def alloc(self, nbytes: int) -> int:
        return lib().kleidicv_gpu_server_alloc(self.handle, nbytes) or 0

    def free(self, ptr: int):
        lib().kleidicv_gpu_server_free(self.handle, ptr)

    def submit(self, request):
        """Returns (error, id)."""
        rid = ctypes.c_uint64()
        err = lib().kleidicv_gpu_server_submit(self.handle, ctypes.byref(request), ctypes.byref(rid))
        return err, rid.value

    def poll(self, capacity=256, timeout_ms=0):
        buf = (Completion * capacity)()
        n = lib().kleidicv_gpu_server_poll(self.handle, buf, capacity, timeout_ms)
        return [(c.id, c.status, c.arrival_s, c.admitted_s, c.completed_s) for c in buf[:n]]

    def now(self) -> float:
        return lib().kleidicv_gpu_server_now(self.handle)

    def drain(self) -> int:
        return lib().kleidicv_gpu_server_drain(self.handle)

    def close(self):
        if self.handle:
            lib().kleidicv_gpu_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        # At interpreter exit the CUDA runtime may already be gone: leave the
        # release to process teardown instead of calling into it.
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


# --- torch helpers ---------------------------------------------------------

def ptr(t):
    return None if t is None else t.data_ptr()


def stride(t):
    return 0 if t is None else t.stride(0) * t.element_size()
