"""Serving loop: requests submitted while earlier batches are on the GPU
(continuous batching) must each give the bytes of the same request run alone
(the plain C-ABI call) and of the CPU oracle; the queue cap answers BUSY; the
pool cap refuses allocations beyond it; drain waits for everything."""
import time

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import __graft_entry__ as ge  # noqa: E402
from oracle import oracle  # noqa: E402

pytestmark = pytest.mark.gpu

kcv = ge.package()


def _mk_requests(rng, n):
    out = []
    for _ in range(n):
        r = rng.random()
        c = int(rng.choice([1, 3, 4]))
        w = int(np.exp(rng.uniform(np.log(32), np.log(700))))
        h = int(np.exp(rng.uniform(np.log(24), np.log(300))))
        if r < 0.6:
            k = int(rng.choice([3, 5, 7, 15]))
            w, h = max(w, k), max(h, k)
            out.append(("gauss", dict(w=w, h=h, c=c, k=k, sigma=float(rng.uniform(0.5, 4.0)),
                                      border=int(rng.choice([1, 2, 3, 4])))))
        elif r < 0.85:
            out.append(("sep", dict(w=w, h=h, c=c, kx=list(rng.integers(0, 5, 5)), ky=list(rng.integers(0, 5, 5)),
                                    border=int(rng.choice([1, 2, 3, 4])))))
        else:
            out.append(("bd", dict(w=max(w, 4), h=max(h, 4), c=c, border=int(rng.choice([1, 2, 3, 4])))))
    return out


def test_continuous_batching_matches_plain_and_oracle():
    rng = np.random.default_rng(44)
    srv = kcv.Server(0, pool_limit_bytes=2 << 30, max_inflight_batches=3, max_batch_requests=16)
    cases = _mk_requests(rng, 60)
    items = []
    for op, s in cases:
        dtype = np.uint16 if op == "sep" else np.uint8
        ow, oh = ((s["w"] + 1) // 2, (s["h"] + 1) // 2) if op == "bd" else (s["w"], s["h"])
        info = np.iinfo(dtype)
        host = rng.integers(0, int(info.max) + 1, (s["h"], s["w"] * s["c"]), dtype=dtype)
        src = torch.from_numpy(host.view(np.int16) if dtype == np.uint16 else host).cuda()
        dst = torch.full((oh, ow * s["c"]), 0x55, dtype=src.dtype, device="cuda")
        alone = torch.full_like(dst, 0x55)
        es = host.dtype.itemsize
        common = (src.data_ptr(), s["w"] * s["c"] * es, dst.data_ptr(), ow * s["c"] * es, s["w"], s["h"], s["c"])
        if op == "gauss":
            req = kcv.make_request(kcv.OP_GAUSSIAN_BLUR_U8, *common, s["k"], s["k"], s["sigma"], s["sigma"],
                                   border_type=s["border"])
            _, want = oracle.gaussian_blur_u8(host, s["w"], s["h"], s["c"], s["k"], s["sigma"], s["border"])
        elif op == "sep":
            req = kcv.make_request(kcv.OP_SEPARABLE_U16, *common, 5, 5, kernel_x=s["kx"], kernel_y=s["ky"],
                                   border_type=s["border"])
            _, want = oracle.separable_filter_2d(host, s["w"], s["h"], s["c"], np.array(s["kx"], np.uint16),
                                                 np.array(s["ky"], np.uint16), s["border"])
        else:
            req = kcv.make_request(kcv.OP_BLUR_AND_DOWNSAMPLE_U8, *common, border_type=s["border"])
            _, want = oracle.blur_and_downsample_u8(host, s["w"], s["h"], s["c"], s["border"])
        items.append(dict(op=op, s=s, src=src, dst=dst, alone=alone, req=req, want=want, dtype=dtype, ow=ow))
    torch.cuda.synchronize()
    ids = {}
    # Arrivals in three waves: later waves arrive while earlier batches run.
    for wave in range(3):
        for i in range(wave, len(items), 3):
            err, rid = srv.submit(items[i]["req"])
            assert err == kcv.OK
            ids[rid] = i
        time.sleep(0.002)
    done = {}
    t_end = time.time() + 30
    while len(done) < len(items) and time.time() < t_end:
        for rid, st, ta, tad, tc in srv.poll(64, timeout_ms=100):
            done[rid] = (st, ta, tad, tc)
    assert srv.drain() == kcv.OK
    assert len(done) == len(items)
    for rid, (st, ta, tad, tc) in done.items():
        assert st == kcv.OK
        assert ta <= tad <= tc
    # Each request alone, through the plain call.
    ctx = kcv.Context.for_torch(0)
    for it in items:
        s = it["s"]
        es = np.dtype(it["dtype"]).itemsize
        args = (it["src"].data_ptr(), s["w"] * s["c"] * es, it["alone"].data_ptr(), it["ow"] * s["c"] * es,
                s["w"], s["h"], s["c"])
        if it["op"] == "gauss":
            e = kcv.gaussian_blur_u8(*args, s["k"], s["k"], s["sigma"], s["sigma"], s["border"], ctx)
        elif it["op"] == "sep":
            e = kcv.separable_filter_2d("u16", *args, s["kx"], 5, s["ky"], 5, s["border"], ctx)
        else:
            e = kcv.blur_and_downsample_u8(args[0], args[1], s["w"], s["h"], args[2], args[3], s["c"], s["border"], ctx)
        assert e == kcv.OK
    assert ctx.synchronize() == kcv.OK
    for i, it in enumerate(items):
        mixed = it["dst"].cpu().numpy()
        alone = it["alone"].cpu().numpy()
        assert np.array_equal(mixed, alone), f"request {i}: mixed result differs from alone"
        want = it["want"].view(np.int16) if it["dtype"] == np.uint16 else it["want"]
        assert np.array_equal(mixed, want), f"request {i}: differs from the oracle"
    ctx.close()
    srv.close()


def test_queue_cap_and_pool_cap():
    srv = kcv.Server(0, pool_limit_bytes=64 << 20, max_inflight_batches=1, max_batch_requests=4, max_queue=2)
    assert srv.alloc(128 << 20) == 0  # beyond the pool cap
    p = srv.alloc(1 << 20)
    assert p != 0
    srv.free(p)
    big = torch.zeros((2000, 4000), dtype=torch.uint8, device="cuda")
    out = torch.zeros_like(big)
    req = kcv.make_request(kcv.OP_GAUSSIAN_BLUR_U8, big.data_ptr(), 4000, out.data_ptr(), 4000, 4000, 2000, 1,
                           21, 21, 3.0, 3.0, border_type=kcv.REFLECT)
    results = [srv.submit(req)[0] for _ in range(12)]
    assert kcv.OK in results
    assert kcv.ERROR_BUSY in results or results.count(kcv.OK) == 12
    assert srv.drain() == kcv.OK
    srv.close()
