"""kleidicv_gpu_gaussian_blur_u8_noalloc against kleidicv_gpu_gaussian_blur_u8
and the CPU oracle.

The allocation-free entry must give the same bytes as the context entry (and
as the oracle) for the requests it serves (two-pass arbitrary-size kernel,
plain copy), on consecutive calls that reuse its one scratch buffer; repeated
calls must leave the device's free memory and torch's allocator untouched;
and it must reject what it does not serve.  This file is collected last so
that it also runs after every other GPU test has used the device.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import __graft_entry__ as ge  # noqa: E402
from oracle import oracle  # noqa: E402
from tests.gpu_harness import _cudart  # noqa: E402

pytestmark = pytest.mark.gpu

kcv = ge.package()


def _image(rng, w, h, c, pad=7):
    host = rng.integers(0, 256, (h, w * c + pad), dtype=np.uint8)
    return torch.from_numpy(host).cuda()


def _both(src, w, h, c, k, sigma, border):
    stream = torch.cuda.current_stream()
    ctx = kcv.Context.for_torch(0)
    got = torch.full((h, w * c + 3), 0xA5, dtype=torch.uint8, device="cuda")
    want = torch.full_like(got, 0xA5)
    e1 = kcv.gaussian_blur_u8_noalloc(src.data_ptr(), src.stride(0), got.data_ptr(), got.stride(0),
                                      w, h, c, k, k, sigma, sigma, border, stream.cuda_stream)
    e2 = kcv.gaussian_blur_u8(src.data_ptr(), src.stride(0), want.data_ptr(), want.stride(0),
                              w, h, c, k, k, sigma, sigma, border, ctx)
    assert ctx.synchronize() == kcv.OK
    ctx.close()
    return e1, e2, got, want


def test_two_calls_in_a_row_match_context_entry():
    rng = np.random.default_rng(11)
    cases = [(997, 613, 3, 31, 0.0), (640, 481, 1, 11, 2.5)]
    srcs = [_image(rng, w, h, c) for (w, h, c, _, _) in cases]
    stream = torch.cuda.current_stream()
    outs = []
    # Two no-alloc calls back to back on one stream (the second reuses the
    # scratch the first just used), then the context entry for each.
    for (w, h, c, k, s), src in zip(cases, srcs):
        dst = torch.full((h, w * c + 3), 0xA5, dtype=torch.uint8, device="cuda")
        err = kcv.gaussian_blur_u8_noalloc(src.data_ptr(), src.stride(0), dst.data_ptr(), dst.stride(0),
                                           w, h, c, k, k, s, s, kcv.REPLICATE, stream.cuda_stream)
        assert err == kcv.OK
        outs.append(dst)
    ctx = kcv.Context.for_torch(0)
    for (w, h, c, k, s), src, got in zip(cases, srcs, outs):
        want = torch.full_like(got, 0xA5)
        err = kcv.gaussian_blur_u8(src.data_ptr(), src.stride(0), want.data_ptr(), want.stride(0),
                                   w, h, c, k, k, s, s, kcv.REPLICATE, ctx)
        assert err == kcv.OK
        assert ctx.synchronize() == kcv.OK
        assert torch.equal(got, want), f"k={k}: {(got != want).sum().item()} bytes differ"
        oerr, owant = oracle.gaussian_blur_u8(src.cpu().numpy(), w, h, c, k, s, kcv.REPLICATE, nthreads=8)
        assert oerr == oracle.OK
        assert np.array_equal(got.cpu().numpy()[:, : w * c], owant), f"k={k}: differs from the oracle"
    ctx.close()


def _free_device_bytes():
    free, total = ctypes.c_size_t(), ctypes.c_size_t()
    assert _cudart().cudaMemGetInfo(ctypes.byref(free), ctypes.byref(total)) == 0
    return free.value


def test_repeated_calls_allocate_nothing():
    """After one warm-up call (which resolves the scratch buffer's address),
    further calls change neither the device's free memory nor torch's
    allocator counters."""
    rng = np.random.default_rng(14)
    w, h, c, k = 1203, 777, 3, 23
    src = _image(rng, w, h, c)
    dst = torch.empty((h, w * c), dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream().cuda_stream

    def call():
        return kcv.gaussian_blur_u8_noalloc(src.data_ptr(), src.stride(0), dst.data_ptr(), dst.stride(0),
                                            w, h, c, k, k, 3.0, 3.0, kcv.REPLICATE, s)

    assert call() == kcv.OK
    torch.cuda.synchronize()
    free0 = _free_device_bytes()
    allocs0 = torch.cuda.memory_stats().get("allocation.all.allocated", 0)
    for _ in range(20):
        assert call() == kcv.OK
    torch.cuda.synchronize()
    assert _free_device_bytes() == free0
    assert torch.cuda.memory_stats().get("allocation.all.allocated", 0) == allocs0
    oerr, want = oracle.gaussian_blur_u8(src.cpu().numpy(), w, h, c, k, 3.0, kcv.REPLICATE, nthreads=8)
    assert oerr == oracle.OK and np.array_equal(dst.cpu().numpy(), want)


def test_copy_kernel_matches():
    # sigma so small that the generated kernel is all centre weight -> copy.
    rng = np.random.default_rng(12)
    w, h, c = 301, 97, 4
    src = _image(rng, w, h, c)
    e1, e2, got, want = _both(src, w, h, c, 13, 0.01, kcv.REPLICATE)
    assert e1 == e2 == kcv.OK
    assert torch.equal(got, want)


def test_oversized_request_is_rejected():
    # ceil16(8192) * 4097 bytes > 32 MiB: RANGE, nothing enqueued.
    w, h, c = 8192, 4097, 1
    src = torch.zeros((h, w), dtype=torch.uint8, device="cuda")
    dst = torch.full_like(src, 0x5A)
    err = kcv.gaussian_blur_u8_noalloc(src.data_ptr(), w, dst.data_ptr(), w, w, h, c, 31, 31, 0.0, 0.0,
                                       kcv.REPLICATE, torch.cuda.current_stream().cuda_stream)
    assert err == kcv.RANGE
    torch.cuda.synchronize()
    assert bool((dst == 0x5A).all())


def test_fused_sizes_and_validation_follow_the_drop_in():
    rng = np.random.default_rng(13)
    w, h, c = 64, 40, 1
    src = _image(rng, w, h, c)
    dst = torch.zeros((h, w), dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    # Sizes the fused kernels compute: not served here.
    assert kcv.gaussian_blur_u8_noalloc(src.data_ptr(), src.stride(0), dst.data_ptr(), w, w, h, c,
                                        5, 5, 0.0, 0.0, kcv.REPLICATE, s) == kcv.NOT_IMPLEMENTED
    # Drop-in validation order: arbitrary sizes need REPLICATE, then pointers.
    assert kcv.gaussian_blur_u8_noalloc(src.data_ptr(), src.stride(0), dst.data_ptr(), w, w, h, c,
                                        11, 11, 0.0, 0.0, kcv.REFLECT, s) == kcv.NOT_IMPLEMENTED
    assert kcv.gaussian_blur_u8_noalloc(None, src.stride(0), dst.data_ptr(), w, w, h, c,
                                        11, 11, 0.0, 0.0, kcv.REPLICATE, s) == kcv.NULL_POINTER
