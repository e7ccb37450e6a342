"""Failure paths on the GPU, made without faulting it: injected allocation
failures and a capped pool give KLEIDICV_ERROR_ALLOCATION (the reference's
answer to a failed workspace malloc), and a bounded device wait that runs out
is reported as KLEIDICV_GPU_ERROR_TIMEOUT with the context still usable."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import __graft_entry__ as ge  # noqa: E402
from oracle import oracle  # noqa: E402

pytestmark = pytest.mark.gpu

kcv = ge.package()


def _img(rng, w, h, c):
    host = rng.integers(0, 256, (h, w * c), dtype=np.uint8)
    return host, torch.from_numpy(host).cuda(), torch.zeros((h, w * c), dtype=torch.uint8, device="cuda")


def _arbitrary(ctx, src, dst, w, h, c, k=31):
    return kcv.gaussian_blur_u8(src.data_ptr(), w * c, dst.data_ptr(), w * c, w, h, c, k, k, 0.0, 0.0,
                                kcv.REPLICATE, ctx)


def test_injected_allocation_failure_then_recovery():
    rng = np.random.default_rng(1)
    w, h, c = 300, 120, 3
    host, src, dst = _img(rng, w, h, c)
    ctx = kcv.Context.for_torch(0)
    ctx.fail_next_allocations(1)
    assert _arbitrary(ctx, src, dst, w, h, c) == kcv.ALLOCATION
    assert ctx.synchronize() == kcv.OK
    assert _arbitrary(ctx, src, dst, w, h, c) == kcv.OK
    assert ctx.synchronize() == kcv.OK
    _, want = oracle.gaussian_blur_u8(host, w, h, c, 31, 0.0, kcv.REPLICATE)
    assert np.array_equal(dst.cpu().numpy(), want)
    ctx.close()


def test_pool_cap_refuses_scratch_and_batch_memory():
    rng = np.random.default_rng(2)
    w, h, c = 400, 300, 4
    _, src, dst = _img(rng, w, h, c)
    ctx = kcv.Context(0, torch.cuda.current_stream().cuda_stream, pool_limit=1024)
    assert _arbitrary(ctx, src, dst, w, h, c) == kcv.ALLOCATION
    # A three-channel request: its tiled-kernel job record (with tensor maps)
    # and work-list exceed the 1 KiB cap (a four-channel 7x7 request would
    # take a 256-byte entry of the streaming kernel's table).
    req = kcv.make_request(kcv.OP_GAUSSIAN_BLUR_U8, src.data_ptr(), w * c, dst.data_ptr(), w * c, w, h, 3, 7, 7,
                           1.5, 1.5, border_type=kcv.REFLECT)
    with pytest.raises(RuntimeError, match="ALLOCATION"):
        kcv.BatchPlan([req], ctx)
    assert ctx.synchronize() == kcv.OK
    ctx.close()


def test_bounded_wait_timeout_is_reported_and_context_survives():
    rng = np.random.default_rng(3)
    ctx = kcv.Context.for_torch(0)
    assert kcv.lib().kleidicv_gpu_selftest_bounded_wait(ctx.handle, 2_000_000) == kcv.OK  # 2 ms
    assert ctx.synchronize() == kcv.ERROR_TIMEOUT
    assert ctx.synchronize() == kcv.OK  # reported once
    w, h, c = 200, 100, 1
    host, src, dst = _img(rng, w, h, c)
    assert kcv.gaussian_blur_u8(src.data_ptr(), w, dst.data_ptr(), w, w, h, c, 5, 5, 0.0, 0.0, kcv.REFLECT,
                                ctx) == kcv.OK
    assert ctx.synchronize() == kcv.OK
    _, want = oracle.gaussian_blur_u8(host, w, h, c, 5, 0.0, kcv.REFLECT)
    assert np.array_equal(dst.cpu().numpy(), want)
    assert kcv.lib().kleidicv_gpu_selftest_bounded_wait(ctx.handle, 0) == kcv.RANGE
    ctx.close()


SHAPES = [(64, 0, 2, 0), (96, 0, 8, 0), (128, 0, 2, 8), (128, 12, 4, 6), (96, 20, 4, 0), (32, 0, 4, 0),
          (64, 0, 4, 8), (128, 0, 2, 6), (96, 0, 2, 0), (64, 0, 2, 8), (128, 0, 8, 0), (64, 0, 8, 6)]


@pytest.mark.parametrize("shape", SHAPES)
def test_forced_tile_shapes_keep_parity(shape):
    """Every shape the autotuner may pick gives the oracle's bytes."""
    rng = np.random.default_rng(4)
    ctx = kcv.Context.for_torch(0)
    assert ctx.set_tile_shape(*shape) == kcv.OK
    cases = [("g", 5, 0.0, 4, kcv.REPLICATE), ("g", 7, 1.5, 4, kcv.REVERSE), ("g", 15, 2.0, 3, kcv.WRAP),
             ("g", 21, 3.0, 1, kcv.REFLECT), ("g", 9, 0.0, 2, kcv.WRAP)]
    for _, k, sigma, c, border in cases:
        w, h = 777, 301
        host, src, dst = _img(rng, w, h, c)
        assert kcv.gaussian_blur_u8(src.data_ptr(), w * c, dst.data_ptr(), w * c, w, h, c, k, k, sigma, sigma,
                                    border, ctx) == kcv.OK
        assert ctx.synchronize() == kcv.OK
        _, want = oracle.gaussian_blur_u8(host, w, h, c, k, sigma, border)
        assert np.array_equal(dst.cpu().numpy(), want), (shape, k, c)
    w, h = 513, 211
    host = rng.integers(0, 65536, (h, w), dtype=np.uint16)
    src = torch.from_numpy(host.view(np.int16)).cuda()
    dst = torch.zeros_like(src)
    kx, ky = [1, 3, 0, 2, 4], [2, 0, 1, 1, 3]
    assert kcv.separable_filter_2d("u16", src.data_ptr(), 2 * w, dst.data_ptr(), 2 * w, w, h, 1, kx, 5, ky, 5,
                                   kcv.WRAP, ctx) == kcv.OK
    assert ctx.synchronize() == kcv.OK
    _, want = oracle.separable_filter_2d(host, w, h, 1, np.array(kx, np.uint16), np.array(ky, np.uint16), kcv.WRAP)
    assert np.array_equal(dst.cpu().numpy().view(np.uint16), want), shape
    host8 = rng.integers(0, 256, (h, w * 3), dtype=np.uint8)
    src8 = torch.from_numpy(host8).cuda()
    ow, oh = (w + 1) // 2, (h + 1) // 2
    dst8 = torch.zeros((oh, ow * 3), dtype=torch.uint8, device="cuda")
    assert kcv.blur_and_downsample_u8(src8.data_ptr(), w * 3, w, h, dst8.data_ptr(), ow * 3, 3, kcv.REVERSE,
                                      ctx) == kcv.OK
    assert ctx.synchronize() == kcv.OK
    _, want8 = oracle.blur_and_downsample_u8(host8, w, h, 3, kcv.REVERSE)
    assert np.array_equal(dst8.cpu().numpy(), want8), shape
    ctx.close()
