"""Batched execution through the C ABI: a plan of uneven requests (every op,
size class, channel count, border and kernel family, plus requests the single
calls reject) must give every image exactly the bytes of the CPU oracle and
every request the status of its single call, with and without a CUDA graph,
on repeated launches."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import __graft_entry__ as ge  # noqa: E402
from oracle import oracle  # noqa: E402
from gpu_harness import device_image, device_output, read_output  # noqa: E402

pytestmark = pytest.mark.gpu

kcv = ge.package()
FIXED = (kcv.REPLICATE, kcv.REFLECT, kcv.WRAP, kcv.REVERSE)


def _case_list(seed=21):
    """(op, spec) pairs; spec holds the host image and the call's arguments."""
    rng = np.random.default_rng(seed)
    cases = []
    for _ in range(40):
        k = int(rng.choice([3, 5, 7, 9, 15, 21]))
        c = int(rng.integers(1, 5))
        w = int(rng.integers(max(k, 8), 400))
        h = int(rng.integers(max(k, 8), 160))
        sigma = 0.0 if rng.random() < 0.3 and k <= 9 else float(rng.uniform(0.5, 4.0))
        border = int(rng.choice(FIXED))
        cases.append(("gauss", dict(w=w, h=h, c=c, k=k, sigma=sigma, border=border, ext=False, bv=0)))
    for k in (11, 13, 31):  # arbitrary sizes: REPLICATE, two-pass kernel
        cases.append(("gauss", dict(w=int(rng.integers(80, 300)), h=int(rng.integers(40, 120)), c=3, k=k,
                                    sigma=float(rng.uniform(1, 6)), border=kcv.REPLICATE, ext=False, bv=0)))
    cases.append(("gauss", dict(w=77, h=33, c=4, k=3, sigma=0.01, border=kcv.REFLECT, ext=False, bv=0)))  # copy
    cases.append(("gauss", dict(w=90, h=41, c=1, k=7, sigma=1.2, border=kcv.CONSTANT, ext=True, bv=17)))
    for dt in ("u8", "u16", "s16"):
        for border in (kcv.REFLECT, kcv.WRAP, kcv.CONSTANT):
            lo, hi = (0, 4) if dt != "s16" else (-4, 4)
            cases.append(("sep", dict(dt=dt, w=int(rng.integers(8, 500)), h=int(rng.integers(8, 120)),
                                      c=int(rng.integers(1, 5)), kx=list(rng.integers(lo, hi + 1, 5)),
                                      ky=list(rng.integers(lo, hi + 1, 5)), border=border,
                                      ext=(border == kcv.CONSTANT or dt == "s16"), bv=17)))
    cases.append(("sep", dict(dt="u16", w=64, h=40, c=1, kx=[60000, 2, 3, 4, 5], ky=[9, 40000, 1, 1, 1],
                              border=kcv.REPLICATE, ext=False, bv=0)))  # saturating taps
    for _ in range(6):
        cases.append(("bd", dict(w=int(rng.integers(4, 600)), h=int(rng.integers(4, 200)), c=int(rng.integers(1, 5)),
                                 border=int(rng.choice(FIXED)), ext=False, bv=0)))
    # Requests the single calls reject.
    cases.append(("gauss", dict(w=50, h=50, c=1, k=4, sigma=0.0, border=kcv.REFLECT, ext=False, bv=0)))
    cases.append(("gauss", dict(w=50, h=50, c=1, k=5, sigma=0.0, border=kcv.CONSTANT, ext=False, bv=0)))
    cases.append(("gauss", dict(w=50, h=50, c=1, k=11, sigma=0.0, border=kcv.REFLECT, ext=False, bv=0)))
    cases.append(("sep", dict(dt="s16", w=50, h=50, c=1, kx=[1] * 5, ky=[1] * 5, border=kcv.REFLECT, ext=False, bv=0)))
    return cases


def _prepare(cases, rng):
    """Uploads inputs, allocates canary-filled outputs, builds the requests and
    the oracle answers."""
    items = []
    for op, s in cases:
        if op == "gauss":
            dtype, ow, oh = np.uint8, s["w"], s["h"]
        elif op == "sep":
            dtype = {"u8": np.uint8, "u16": np.uint16, "s16": np.int16}[s["dt"]]
            ow, oh = s["w"], s["h"]
        else:
            dtype, ow, oh = np.uint8, (s["w"] + 1) // 2, (s["h"] + 1) // 2
        info = np.iinfo(dtype)
        host = rng.integers(info.min, int(info.max) + 1, (s["h"], s["w"] * s["c"] + s.get("pad", 5)), dtype=dtype)
        sbuf, sptr, sstride = device_image(torch, host)
        dbuf, dptr, dstride = device_output(torch, oh, ow * s["c"], dtype, pad_elems=3)
        if op == "gauss":
            req = kcv.make_request(kcv.OP_GAUSSIAN_BLUR_U8, sptr, sstride, dptr, dstride, s["w"], s["h"], s["c"],
                                   s["k"], s["k"], s["sigma"], s["sigma"], border_type=s["border"],
                                   border_value=s["bv"], allow_extensions=s["ext"])
            werr, want = oracle.gaussian_blur_u8(host, s["w"], s["h"], s["c"], s["k"], s["sigma"], s["border"],
                                                 ext=s["ext"], border_value=s["bv"])
        elif op == "sep":
            code = {"u8": kcv.OP_SEPARABLE_U8, "u16": kcv.OP_SEPARABLE_U16, "s16": kcv.OP_SEPARABLE_S16}[s["dt"]]
            req = kcv.make_request(code, sptr, sstride, dptr, dstride, s["w"], s["h"], s["c"], 5, 5,
                                   kernel_x=s["kx"], kernel_y=s["ky"], border_type=s["border"],
                                   border_value=s["bv"], allow_extensions=s["ext"])
            if s["dt"] == "s16" and not s["ext"]:
                werr, want = kcv.NOT_IMPLEMENTED, None
            else:
                werr, want = oracle.separable_filter_2d(host, s["w"], s["h"], s["c"], np.array(s["kx"], dtype),
                                                        np.array(s["ky"], dtype), s["border"], ext=s["ext"],
                                                        border_value=s["bv"])
        else:
            req = kcv.make_request(kcv.OP_BLUR_AND_DOWNSAMPLE_U8, sptr, sstride, dptr, dstride, s["w"], s["h"],
                                   s["c"], border_type=s["border"], allow_extensions=s["ext"])
            werr, want = oracle.blur_and_downsample_u8(host, s["w"], s["h"], s["c"], s["border"])
        items.append(dict(req=req, sbuf=sbuf, dbuf=dbuf, dstride=dstride, rows=oh, elems=ow * s["c"],
                          dtype=dtype, werr=werr, want=want))
    return items


def _check(items, statuses):
    for i, it in enumerate(items):
        assert statuses[i] == it["werr"], f"request {i}: status {statuses[i]} != {it['werr']}"
        if it["werr"] != kcv.OK:
            continue
        got, pad_ok = read_output(it["dbuf"], it["rows"], it["elems"], it["dtype"], it["dstride"])
        assert pad_ok, f"request {i}: wrote outside its image"
        assert np.array_equal(got, it["want"]), f"request {i}: {(got != it['want']).sum()} elements differ"


def _refill(items):
    for it in items:
        it["dbuf"].fill_(0xA5)


@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_plan_matches_oracle(use_graph):
    rng = np.random.default_rng(5)
    items = _prepare(_case_list(), rng)
    ctx = kcv.Context.for_torch(0)
    plan = kcv.BatchPlan([it["req"] for it in items], ctx)
    assert plan.tile_count() > 0
    for _ in range(2):  # the second launch replays the graph
        _refill(items)
        assert plan.launch(use_graph) == kcv.OK
        assert ctx.synchronize() == kcv.OK
        _check(items, plan.statuses)
    plan.close()
    ctx.close()


def test_batch_submit_matches_oracle():
    rng = np.random.default_rng(6)
    items = _prepare(_case_list(seed=22), rng)
    ctx = kcv.Context.for_torch(0)
    err, statuses = kcv.batch_submit([it["req"] for it in items], ctx)
    assert err == kcv.OK
    assert ctx.synchronize() == kcv.OK
    _check(items, statuses)
    ctx.close()


def test_batch_of_nothing_and_only_rejects():
    ctx = kcv.Context.for_torch(0)
    plan = kcv.BatchPlan([], ctx)
    assert plan.tile_count() == 0
    assert plan.launch(True) == kcv.OK
    bad = kcv.make_request(kcv.OP_GAUSSIAN_BLUR_U8, None, 64, None, 64, 64, 64, 1, 5, 5, 0.0, 0.0,
                           border_type=kcv.REFLECT)
    plan2 = kcv.BatchPlan([bad], ctx)
    assert plan2.statuses == [kcv.NULL_POINTER]
    assert plan2.launch(False) == kcv.OK
    assert ctx.synchronize() == kcv.OK
    plan.close()
    plan2.close()
    ctx.close()


def test_uneven_batch_512_all_outputs():
    """The 512-image uneven batch (seed 2: w 64-4096 and h 64-2160 log-uniform,
    C {1,3,4}, k {3,5,7,15}, sigma 0.5-4, random border), one graph launch of
    one plan: every output equals the oracle's."""
    rng = np.random.default_rng(2)
    ctx = kcv.Context.for_torch(0)
    items = []
    for _ in range(512):
        w = int(round(float(np.exp(rng.uniform(np.log(64), np.log(4096))))))
        h = int(round(float(np.exp(rng.uniform(np.log(64), np.log(2160))))))
        c = int(rng.choice([1, 3, 4]))
        k = int(rng.choice([3, 5, 7, 15]))
        sigma = float(rng.uniform(0.5, 4.0))
        border = int(rng.choice([kcv.REPLICATE, kcv.REFLECT, kcv.WRAP, kcv.REVERSE]))
        host = rng.integers(0, 256, (h, w * c), dtype=np.uint8)
        src = torch.from_numpy(host).cuda()
        dst = torch.zeros_like(src)
        items.append((host, src, dst, w, h, c, k, sigma, border))
    reqs = [kcv.make_request(kcv.OP_GAUSSIAN_BLUR_U8, it[1].data_ptr(), it[3] * it[5], it[2].data_ptr(),
                             it[3] * it[5], it[3], it[4], it[5], it[6], it[6], it[7], it[7], border_type=it[8])
            for it in items]
    plan = kcv.BatchPlan(reqs, ctx)
    assert all(st == kcv.OK for st in plan.statuses)
    assert plan.launch(True) == kcv.OK
    assert ctx.synchronize() == kcv.OK
    bad = []
    for i, it in enumerate(items):
        e, want = oracle.gaussian_blur_u8(it[0], it[3], it[4], it[5], it[6], it[7], it[8], nthreads=16)
        if e != 0 or not np.array_equal(it[2].cpu().numpy(), want):
            bad.append(i)
    plan.close()
    ctx.close()
    assert not bad, f"{len(bad)} of 512 outputs differ, first {bad[:5]}"


@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_of_downsamples_pyramid_tables(use_graph):
    """A plan of blur-and-downsample requests only (one pyramid-kernel launch
    per channel count over a device entry table): 70 requests of every
    channel count and border, aligned and unaligned sources, odd sizes down
    to 1x1, on two launches."""
    rng = np.random.default_rng(31)
    cases = []
    for i in range(70):
        w, c = (int(rng.integers(1, 900)) if i % 9 else 1), int(rng.integers(1, 5))
        pad = (-(w * c)) % 16 if i % 2 else 5  # odd requests: 16-byte rows (the kernel's staged strips)
        cases.append(("bd", dict(w=w, h=int(rng.integers(1, 300)), c=c, border=int(rng.choice(FIXED)), ext=False,
                                 bv=0, pad=pad)))
    items = _prepare(cases, rng)
    ctx = kcv.Context.for_torch(0)
    plan = kcv.BatchPlan([it["req"] for it in items], ctx)
    for _ in range(2):
        _refill(items)
        assert plan.launch(use_graph) == kcv.OK
        assert ctx.synchronize() == kcv.OK
        _check(items, plan.statuses)
    plan.close()
    ctx.close()
