"""Benchmark of the GB300 separable-filter library on the plain drop-in sweep.

One step is one pass of the sweep over device-resident synthetic images (seed 1):

  * gaussian_blur_u8     3840x2160x4 u8, 7x7, sigma 1.5, border REVERSE
  * separable_filter_2d  3840x2160x1 u16 and s16, 5x5 taps drawn from seed 1,
                         borders REFLECT, WRAP and CONSTANT (border value 17,
                         through the _ex extension: the drop-in entry returns
                         NOT_IMPLEMENTED for CONSTANT, as KleidiCV does)

Every image is half uniform noise and half a smooth gradient, with step edges
1-7 px from every border.  Two buffer sets (531 MB, more than 4x the 129 MB L2)
alternate between steps, so no step reads what the previous one left in L2.

Printed: one JSON line (rank 0).  `value` is output Mpix/s of the whole job
(all ranks) with inputs resident in HBM; `e2e` is the same metric through the
public C-ABI calls with pinned HOST buffers, the host<->device copies inside
the timed region; `roofline` is the 4K RGBA Gaussian kernel against the
measured HBM copy bandwidth; `cpu_baseline` is the reference's CPU path
(kleidicv_thread_* on all host cores; the CPU restatement oracle/kcv_oracle.c
where the reference is not available) on the same inputs, whose output is also
compared byte for byte with the GPU's.

`--impl reference` times the reference's own CPU path alone: KleidiCV and
kleidicv_thread, built from their sources on an AArch64 host (oracle/Makefile,
target `refnative`), driven by a persistent pool of all host threads, on the
same images.  On a host where the reference cannot be built the CPU
restatement stands in, and the line says so.

Multi-GPU: images are independent, so N ranks run N replicas of the sweep with
no collective on the data path ("replicas only"); the step time is the max over
ranks and `value` counts the pixels of all ranks.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

W, H = 3840, 2160
REF_BUDGET_S = 120.0  # timed seconds the reference arm may spend on its K steps
BORDER_VALUE = 17
N_SETS = 2
METRIC = "Mpix/s"
WORKLOAD = ("plain drop-in sweep (seed 1): gaussian_blur_u8 3840x2160x4 7x7 sigma 1.5 REVERSE; "
            "separable_filter_2d u16 and s16 3840x2160x1 5x5, REFLECT / WRAP / CONSTANT(17)")
GAUSS_BYTES = 2 * W * H * 4  # algorithmic bytes of one Gaussian launch: read + write once


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    ap.add_argument("--e2e-steps", type=int, default=40)
    ap.add_argument("--cpu-passes", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sections", default="c1,batched,pyramid,lk_pyramid,sobel,median,thread_api,serving",
                    help="extra measurements added to the line (comma list, or 'none')")
    ap.add_argument("--profile-op", choices=("gauss", "u16", "s16", "blurdown", "sobel", "arbitrary", "median5",
                                             "median15", "lk"), default=None,
                    help="run one workload 3 times on cuda:0 and exit (a small command for profiler captures): "
                         "the sweep's Gaussian / u16 REFLECT / s16 REFLECT call, blur_and_downsample_u8 of a "
                         "4096x4096x1 image, the d/dx Sobel of a 3840x2160x1 image, a 31x31 sigma 5 Gaussian "
                         "(REPLICATE, the generic two-pass kernel) of a 3840x2160x1 image, the 5x5 / 15x15 u8 "
                         "median of a 1920x1080x1 image, or the 4-level LK pyramid of a 1920x1080x1 image")
    ap.add_argument("--profile-range", type=int, default=0,
                    help="with --profile-op: N calls over rotating buffer sets larger than twice the L2, between "
                         "cudaProfilerStart and cudaProfilerStop (an ncu --replay-mode range window that also "
                         "holds the write-back of earlier calls' outputs)")
    ap.add_argument("--serving-seconds", type=float, default=60.0)
    ap.add_argument("--serving-high-seconds", type=float, default=10.0)
    ap.add_argument("--serving-inflight", type=int, default=3)
    ap.add_argument("--serving-batch-mb", type=int, default=0, help="work budget per batch in MiB (0: none)")
    ap.add_argument("--serving-rate", type=float, default=2000.0)
    return ap.parse_args()


# ----------------------------------------------------------------------------
# Synthetic inputs
# ----------------------------------------------------------------------------

def make_image(rng, width, height, channels, lo, hi, dtype):
    """Left half uniform noise, right half a smooth horizontal+vertical
    gradient; a band of 1-7 px along every border holds a different level, so
    each border has a step edge at that distance."""
    span = hi - lo
    img = np.empty((height, width, channels), np.float64)
    img[:, : width // 2] = rng.integers(lo, hi + 1, (height, width // 2, channels))
    gx = np.linspace(0.0, 1.0, width - width // 2)[None, :, None]
    gy = np.linspace(0.0, 1.0, height)[:, None, None]
    img[:, width // 2:] = lo + span * (0.15 + 0.35 * gx + 0.35 * gy)
    for side in range(4):
        d = int(rng.integers(1, 8))
        level = lo + span * float(rng.uniform(0.05, 0.95))
        if side == 0:
            img[:d] = level
        elif side == 1:
            img[-d:] = level
        elif side == 2:
            img[:, :d] = level
        else:
            img[:, -d:] = level
    return np.clip(np.rint(img), lo, hi).astype(dtype).reshape(height, width * channels)


ROOFLINE_EVERY = 8  # timed steps per event-bracketed Gaussian launch


def make_calls():
    """The seven calls of one sweep step: (name, kind, args) with host inputs."""
    rng = np.random.default_rng(1)
    calls = []
    g = make_image(rng, W, H, 4, 0, 255, np.uint8)
    calls.append(dict(name="gaussian_blur_u8 RGBA 7x7 s1.5 REVERSE", op="gauss", dtype="u8",
                      channels=4, src=g, ksize=7, sigma=1.5, border=4, bv=None))
    taps = {
        "u16": (rng.integers(0, 5, 5), rng.integers(0, 5, 5)),
        "s16": (rng.integers(-4, 5, 5), rng.integers(-4, 5, 5)),
    }
    imgs = {
        "u16": make_image(rng, W, H, 1, 0, 65535, np.uint16),
        "s16": make_image(rng, W, H, 1, -32768, 32767, np.int16),
    }
    for dt in ("u16", "s16"):
        for border, bname in ((2, "REFLECT"), (3, "WRAP"), (0, "CONSTANT(17)")):
            calls.append(dict(name=f"separable_filter_2d {dt} 5x5 {bname}", op="sep", dtype=dt,
                              channels=1, src=imgs[dt], kx=taps[dt][0], ky=taps[dt][1],
                              border=border, bv=BORDER_VALUE if border == 0 else None))
    return calls, {k: (list(map(int, a)), list(map(int, b))) for k, (a, b) in taps.items()}


def out_pixels(calls):
    return sum(W * H for _ in calls)


def algorithmic_bytes(calls):
    return sum(2 * c["src"].nbytes for c in calls)


# ----------------------------------------------------------------------------
# GPU arm
# ----------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons (100 ms period)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        import threading

        self.lines = []
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={device_index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            return
        self.reader = threading.Thread(target=self._read, daemon=True)
        self.reader.start()

    def _read(self):
        for line in self.proc.stdout:
            if line.strip():
                self.lines.append((time.time(), [f.strip() for f in line.split(",")]))

    def stop(self):
        if self.proc is None:
            return
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            self.proc.wait()
        self.reader.join(timeout=5)

    def summary(self, t_start, t_stop):
        if not self.lines:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        window = [f for ts, f in self.lines if t_start - 0.15 <= ts <= t_stop + 0.15]
        where = "timed region"
        if not window:
            window = [f for _, f in self.lines]
            where = "whole run (timed region shorter than the sampling period)"
        sm = [float(f[1]) for f in window if f[1].replace(".", "").isdigit()]
        mx = [float(f[2]) for f in window if f[2].replace(".", "").isdigit()]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({names[k] for f in window for k in range(4)
                          if len(f) > 5 + k and f[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(window), "window": where}


def measured_hbm_peak():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_traffic():
    """dram__bytes_read.sum + dram__bytes_write.sum per launch of the Gaussian
    kernel, from the committed ncu summary (None if absent)."""
    p = os.path.join(REPO, "profiles", "gauss8_gauss7_rgba_4k.md")
    try:
        with open(p) as f:
            for line in f:
                if line.startswith("traffic_bytes_per_launch:"):
                    return int(line.split(":", 1)[1].strip())
    except (OSError, ValueError):
        pass
    return None


def max_over_ranks(x: float) -> float:
    """Largest value of x over the ranks (a timing: the slowest rank sets the
    job's time).  NCCL reduces on the GPU, gloo on the host; one rank returns x."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, world: int, ms_per_step: float) -> float:
    """Units per second of the whole job: every rank processes units_per_rank
    per step (replicas), in the slowest rank's step time."""
    return world * units_per_rank / (ms_per_step * 1e-3)


def run_gpu(args, rank, world, calls, taps):
    import torch
    import __graft_entry__ as ge

    kcv = ge.package()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    ctx = kcv.Context(local, stream.cuda_stream)

    def to_dev(a):
        # u16 images travel as int16 bits: only the pointer reaches the library.
        return torch.from_numpy(a.view(np.int16) if a.dtype == np.uint16 else a).to(dev)

    sets = []
    for _ in range(N_SETS):
        s = []
        for c in calls:
            src = to_dev(c["src"])
            dst = torch.empty_like(src)
            s.append((src, dst))
        sets.append(s)

    def issue(c, src_ptr, src_stride, dst_ptr, dst_stride):
        if c["op"] == "gauss":
            err = kcv.gaussian_blur_u8(src_ptr, src_stride, dst_ptr, dst_stride, W, H, c["channels"],
                                       c["ksize"], c["ksize"], c["sigma"], c["sigma"], c["border"],
                                       ctx, border_value=c["bv"])
        else:
            err = kcv.separable_filter_2d(c["dtype"], src_ptr, src_stride, dst_ptr, dst_stride, W, H,
                                          c["channels"], c["kx"], 5, c["ky"], 5, c["border"], ctx,
                                          border_value=c["bv"])
        if err != kcv.OK:
            raise RuntimeError(f"{c['name']}: {kcv.ERROR_NAMES.get(err, err)}")

    lib = kcv.lib()

    def bind(c, src_ptr, src_stride, dst_ptr, dst_stride):
        """The same C-ABI call as issue(), with its arguments (pointers, strides,
        tap arrays) converted once, so that the timed loop spends almost no
        host time per call: a slow host cannot leave the GPU waiting."""
        h = ctx.handle
        if c["op"] == "gauss":
            fn, args = lib.kleidicv_gpu_gaussian_blur_u8, (
                src_ptr, src_stride, dst_ptr, dst_stride, W, H, c["channels"], c["ksize"], c["ksize"],
                c["sigma"], c["sigma"], c["border"], h)
        else:
            ct = {"u16": ctypes.c_uint16, "s16": ctypes.c_int16}[c["dtype"]]
            kx = (ct * 5)(*[int(v) for v in c["kx"]])
            ky = (ct * 5)(*[int(v) for v in c["ky"]])
            head = (src_ptr, src_stride, dst_ptr, dst_stride, W, H, c["channels"], kx, 5, ky, 5, c["border"])
            if c["dtype"] == "s16":
                fn, args = lib.kleidicv_gpu_separable_filter_2d_s16_ex, head + (c["bv"] or 0, h)
            elif c["bv"] is None:
                fn, args = lib.kleidicv_gpu_separable_filter_2d_u16, head + (h,)
            else:
                fn, args = lib.kleidicv_gpu_separable_filter_2d_u16_ex, head + (c["bv"], h)
        return lambda: fn(*args)

    bound = [[bind(c, src.data_ptr(), src.stride(0) * src.element_size(), dst.data_ptr(),
                   dst.stride(0) * dst.element_size()) for c, (src, dst) in zip(calls, sets[k])]
             for k in range(N_SETS)]

    def step(i, evs=None, only=None):
        """One sweep step; evs[ci] = (start, end) events recorded around call ci
        (for the calls in `only`, or all): an event between two calls also
        stops the next call from starting while the previous one drains."""
        for ci, call in enumerate(bound[i % N_SETS]):
            timed = evs is not None and (only is None or ci in only)
            if timed:
                evs[ci][0].record(stream)
            err = call()
            if timed:
                evs[ci][1].record(stream)
            if err != kcv.OK:
                raise RuntimeError(f"{calls[ci]['name']}: {kcv.ERROR_NAMES.get(err, err)}")

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    sampler = ClockSampler(local)
    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()
    if ctx.synchronize() != kcv.OK:
        raise RuntimeError("warm-up failed")

    per_call = [[] for _ in calls]
    ev_calls = [[(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                 for _ in calls] for _ in range(args.steps)]
    t_begin, t_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    launches0 = ctx.launch_count()
    wall0 = time.time()
    t_begin.record(stream)
    # The Gaussian (the roofline's kernel) is bracketed by events on every
    # eighth step: the events sample its duration live in the timed region
    # while leaving the other steps back to back.
    for i in range(args.steps):
        if i % ROOFLINE_EVERY == 0:
            step(i, ev_calls[i], only=(0,))
        else:
            step(i)
    t_end.record(stream)
    torch.cuda.synchronize()
    wall1 = time.time()
    barrier()
    launches = ctx.launch_count() - launches0
    sampler.stop()
    if ctx.synchronize() != kcv.OK:
        raise RuntimeError("timed region failed")
    for i in range(0, args.steps, ROOFLINE_EVERY):
        per_call[0].append(ev_calls[i][0][0].elapsed_time(ev_calls[i][0][1]))
    # Every call timed on its own (outside the timed region), for the breakdown.
    n_iso = min(args.steps, 200)
    for i in range(n_iso):
        step(i, ev_calls[i])
    torch.cuda.synchronize()
    for i in range(n_iso):
        for ci in range(1, len(calls)):
            per_call[ci].append(ev_calls[i][ci][0].elapsed_time(ev_calls[i][ci][1]))
    ms_total = max_over_ranks(t_begin.elapsed_time(t_end))
    ms_step = ms_total / args.steps
    # The Gaussian back to back (outside the timed region): 100 launches over
    # the rotating buffer sets between two events, i.e. its steady-state
    # duration without the per-launch ramp that the events above include.
    b0, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    b0.record(stream)
    for i in range(100):
        if bound[i % N_SETS][0]() != kcv.OK:
            raise RuntimeError("back-to-back Gaussian failed")
    b1.record(stream)
    torch.cuda.synchronize()
    gauss_b2b_ms = b0.elapsed_time(b1) / 100

    # ---- end to end through the public calls with pinned host buffers.  A
    # three-stream pipeline: the upload of call i+1 and the download of call
    # i-1 overlap the filter of call i (events order each buffer's reuse; the
    # two device buffer sets alternate between steps).
    hsrc = [torch.from_numpy(c["src"].view(np.int16) if c["src"].dtype == np.uint16 else c["src"])
            .pin_memory() for c in calls]
    hdst = [torch.empty_like(h).pin_memory() for h in hsrc]
    h2d = sum(h.numel() * h.element_size() for h in hsrc)
    d2h = sum(h.numel() * h.element_size() for h in hdst)
    up, down = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    comp = stream
    nc = len(calls)
    ev = lambda: torch.cuda.Event()  # noqa: E731
    # per (set, call): uploaded, computed, downloaded
    uploaded = [[ev() for _ in calls] for _ in range(N_SETS)]
    computed = [[ev() for _ in calls] for _ in range(N_SETS)]
    downloaded = [[None] * nc for _ in range(N_SETS)]
    src_free = [[None] * nc for _ in range(N_SETS)]

    def e2e_step(i):
        k = i % N_SETS
        for ci, (c, hs, hd) in enumerate(zip(calls, hsrc, hdst)):
            src, dst = sets[k][ci]
            with torch.cuda.stream(up):
                if src_free[k][ci] is not None:
                    up.wait_event(src_free[k][ci])
                src.copy_(hs, non_blocking=True)
                uploaded[k][ci].record(up)
            comp.wait_event(uploaded[k][ci])
            if downloaded[k][ci] is not None:
                comp.wait_event(downloaded[k][ci])
            issue(c, src.data_ptr(), src.stride(0) * src.element_size(), dst.data_ptr(),
                  dst.stride(0) * dst.element_size())
            computed[k][ci].record(comp)
            src_free[k][ci] = computed[k][ci]
            with torch.cuda.stream(down):
                down.wait_event(computed[k][ci])
                hd.copy_(dst, non_blocking=True)
                e = ev()
                e.record(down)
                downloaded[k][ci] = e

    e2e_n = max(1, min(args.e2e_steps, args.steps))
    for i in range(3):
        e2e_step(i)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    e0.record(up)
    comp.wait_event(e0)
    down.wait_event(e0)
    for i in range(e2e_n):
        e2e_step(i)
    for st_ in (up, comp):
        down.wait_stream(st_)
    e1.record(down)
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks(e0.elapsed_time(e1) / e2e_n)
    if ctx.synchronize() != kcv.OK:
        raise RuntimeError("end-to-end run failed")

    result = dict(ms_step=ms_step, per_call=[statistics.mean(v) for v in per_call], gauss_b2b_ms=gauss_b2b_ms,
                  launches=launches, e2e_ms=e2e_ms, h2d=h2d, d2h=d2h,
                  clocks=sampler.summary(wall0, wall1),
                  outputs=[hd.numpy() for hd in hdst] if rank == 0 else None)
    return result, (lambda: (ctx.close()))


# ----------------------------------------------------------------------------
# CPU paths: the reference itself (KleidiCV + kleidicv_thread, built natively on
# an AArch64 host by oracle/Makefile) when it is available, else the CPU
# restatement of its algorithm (oracle/kcv_oracle.c).  Both use every host core.
# ----------------------------------------------------------------------------

def cpu_pass(calls, nthreads, keep=False, rows=H):
    """One pass of the sweep through the CPU restatement; `rows` < H filters the
    top `rows` rows of every image as an image of that height (a bounded sample)."""
    from oracle import oracle

    outs = []
    for c in calls:
        if c["op"] == "gauss":
            err, out = oracle.gaussian_blur_u8(c["src"], W, rows, c["channels"], c["ksize"], c["sigma"],
                                               c["border"], nthreads=nthreads)
        else:
            ext = c["bv"] is not None
            err, out = oracle.separable_filter_2d(c["src"], W, rows, c["channels"], np.array(c["kx"]),
                                                  np.array(c["ky"]), c["border"], ext=ext,
                                                  border_value=c["bv"] or 0, nthreads=nthreads)
        if err != oracle.OK:
            raise RuntimeError(f"oracle {c['name']}: error {err}")
        if keep:
            outs.append(out)
    return outs


REF_STANDIN = ("the reference implements 3 of the 7 sweep calls (the Gaussian, u16 REFLECT, u16 WRAP); for the "
               "u16 CONSTANT and the three s16 calls it returns NOT_IMPLEMENTED, so each of those steps runs the "
               "u16 call of the same shape and border class instead (CONSTANT -> REFLECT, s16 -> u16), keeping "
               "7 calls of the same sizes per step")


def ref_plan(calls):
    """The 7 reference calls of one step: (index of the GPU call whose output it
    reproduces or None, call dict to run)."""
    u16 = {c["border"]: c for c in calls if c["op"] == "sep" and c["dtype"] == "u16"}
    plan = []
    for i, c in enumerate(calls):
        if c["op"] == "gauss":
            plan.append((i, c))
        elif c["dtype"] == "u16" and c["bv"] is None:
            plan.append((i, c))
        else:
            plan.append((None, u16[c["border"] if c["border"] in (2, 3) else 2]))
    return plan


def ref_pass(plan, pool, keep=False, rows=H):
    """One pass of the reference plan through kleidicv_thread_* on `pool`."""
    from oracle import refimpl

    outs = {}
    for idx, c in plan:
        if c["op"] == "gauss":
            err, out = refimpl.gaussian_blur_u8(c["src"], W, rows, c["channels"], c["ksize"], c["sigma"],
                                                c["border"], pool=pool)
        else:
            dt = c["src"].dtype
            err, out = refimpl.separable_filter_2d(c["src"], W, rows, c["channels"], np.array(c["kx"], dt),
                                                   np.array(c["ky"], dt), c["border"], pool=pool)
        if err != 0:
            raise RuntimeError(f"reference {c['name']}: error {err}")
        if keep and idx is not None:
            outs[idx] = out
    return outs


def reference_cpu():
    """(refimpl module, host info) when the reference library loads here, else (None, reason)."""
    from oracle import refimpl

    why = refimpl.status()
    if why is not None:
        return None, why
    return refimpl, refimpl.host_info()


def _timed_passes(fn, passes):
    times = []
    for _ in range(passes):
        t0 = time.perf_counter()
        fn()
        times.append(time.perf_counter() - t0)
    return statistics.median(times)


def cpu_baseline(calls, passes, outputs=None):
    """The CPU path on the same inputs: the reference (kleidicv_thread on a
    persistent pool of all host cores) when it is available, else the C
    restatement.  Also compares its outputs with the GPU's, byte for byte."""
    from oracle import oracle

    cores = os.cpu_count() or 1
    ref, info = reference_cpu()
    if ref is not None:
        plan = ref_plan(calls)
        pool = ref.Pool(cores)
        try:
            outs = ref_pass(plan, pool, keep=True)  # also warms the pages
            exact = None
            if outputs is not None:
                exact = all(np.array_equal(outs[i].view(np.uint8), outputs[i].view(np.uint8)) for i in outs)
            sec = _timed_passes(lambda: ref_pass(plan, pool), max(passes, 10))
        finally:
            pool.close()
        return dict(value=round(out_pixels(calls) / sec / 1e6, 2), unit=METRIC, cores=cores, kind="reference",
                    sample=f"{max(passes, 10)} full passes (median) of 7 reference calls on 3840x2160 images "
                           f"with {cores} threads: kleidicv_thread_* on a persistent std::thread pool; "
                           + REF_STANDIN,
                    host=info, exact_calls=sorted(outs)), exact
    oracle.build()
    outs = cpu_pass(calls, cores, keep=True)
    exact = None
    if outputs is not None:
        exact = all(np.array_equal(a.view(np.uint8), b.view(np.uint8)) for a, b in zip(outs, outputs))
    sec = _timed_passes(lambda: cpu_pass(calls, cores), passes)
    return dict(value=round(out_pixels(calls) / sec / 1e6, 2), unit=METRIC, cores=cores, kind="port",
                sample=f"{passes} full passes of the 7-call sweep (median) with {cores} threads; "
                       f"CPU restatement oracle/kcv_oracle.c (scalar C, -O3); the reference is not "
                       f"available here: {info}"), exact


# ----------------------------------------------------------------------------
# Further configurations of the workload description, reported beside the
# headline sweep (rank 0, one GPU): the plain 1080p call, the uneven batch,
# the pyramids and the serving loop.
# ----------------------------------------------------------------------------

def _events_time(torch, stream, fn, reps):
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(stream)
    for i in range(reps):
        fn(i)
    b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def section_c1(torch, kcv, ctx, stream):
    """1920x1080x1 u8, 5x5 binomial (sigma 0), REPLICATE, row stride w+64, seed 0."""
    from oracle import oracle

    w, h, stride = 1920, 1080, 1920 + 64
    rng = np.random.default_rng(0)
    host = rng.integers(0, 256, (h, stride), dtype=np.uint8)
    nb = 40  # 40 x 2 x 2.1 MB > L2
    srcs = [torch.from_numpy(host).cuda() for _ in range(nb)]
    dsts = [torch.zeros((h, stride), dtype=torch.uint8, device="cuda") for _ in range(nb)]

    def call(i):
        e = kcv.gaussian_blur_u8(srcs[i % nb].data_ptr(), stride, dsts[i % nb].data_ptr(), stride, w, h, 1,
                                 5, 5, 0.0, 0.0, kcv.REPLICATE, ctx)
        assert e == kcv.OK, e

    for i in range(5):
        call(i)
    ms = _events_time(torch, stream, call, 200)
    _, want = oracle.gaussian_blur_u8(host, w, h, 1, 5, 0.0, kcv.REPLICATE,
                                      dst=np.zeros((h, stride), np.uint8))
    got = dsts[0].cpu().numpy()
    return {"config": "1920x1080x1 u8 5x5 sigma 0 REPLICATE, stride w+64, seed 0",
            "us_per_call": round(ms * 1e3, 2), "mpix_s": round(w * h / (ms * 1e-3) / 1e6, 1),
            "hbm_gbs": round(2 * w * h / (ms * 1e-3) / 1e9, 1),
            "bit_exact_vs_oracle": bool(np.array_equal(got[:, :w], want[:, :w]))}


def section_sobel(torch, kcv, ctx, stream, cores):
    """Sobel 3x3 d/dx and d/dy, u8 -> s16 (REPLICATE), 3840x2160 with 1 and 4
    channels, seed 5: per-call time, HBM rate (1 byte read + 2 written per
    element) against the measured copy bandwidth, and bit-exactness against
    the CPU oracle."""
    from oracle import oracle

    peak, peak_kind = measured_hbm_peak()
    rng = np.random.default_rng(5)
    out = {"config": "3840x2160 u8 -> s16, REPLICATE, seed 5; rotating buffer sets > 2x L2",
           "peak_source": f"{peak_kind} hbm_gbs"}
    for c in (1, 4):
        w, h = 3840, 2160
        host = rng.integers(0, 256, (h, w * c), dtype=np.uint8)
        per_set = 3 * w * h * c
        nb = max(2, -(-300_000_000 // per_set))  # > 2x the 129 MB L2
        srcs = [torch.from_numpy(host).cuda() for _ in range(nb)]
        dsts = [torch.empty((h, w * c), dtype=torch.int16, device="cuda") for _ in range(nb)]
        for name, fn, horizontal in (("dx", kcv.sobel_3x3_horizontal_s16_u8, True),
                                     ("dy", kcv.sobel_3x3_vertical_s16_u8, False)):
            def call(i, fn=fn):
                e = fn(srcs[i % nb].data_ptr(), w * c, dsts[i % nb].data_ptr(), 2 * w * c, w, h, c, ctx)
                assert e == kcv.OK, e

            for i in range(5):
                call(i)
            ms = _events_time(torch, stream, call, 100)
            call(0)
            torch.cuda.synchronize()
            _, want = oracle.sobel_3x3_s16_u8(host, w, h, c, horizontal, nthreads=cores)
            gbs = per_set / (ms * 1e-3) / 1e9
            out[f"{name}_c{c}"] = {"us_per_call": round(ms * 1e3, 2),
                                   "mpix_s": round(w * h / (ms * 1e-3) / 1e6, 1),
                                   "hbm_gbs": round(gbs, 1), "frac": round(gbs / peak, 4),
                                   "bit_exact_vs_oracle": bool(np.array_equal(dsts[0].cpu().numpy(), want))}
        del srcs, dsts
    return out


def section_thread_api(torch, kcv, cores):
    """kleidicv_gpu_thread_gaussian_blur_u8 (KleidiCV's threaded-API contract:
    host images, caller's scheduler, synchronous) on 3840x2160x4, 7x7, sigma
    1.5, REVERSE, seed 1: host wall time per call from pageable and from
    pinned host images, with the library's worker pool of 1 and of all host
    threads driving the packing and unpacking."""
    import time as _t

    w, h, c = 3840, 2160, 4
    rng = np.random.default_rng(1)
    host = rng.integers(0, 256, (h, w * c), dtype=np.uint8)
    out = {"config": "3840x2160x4 u8 7x7 sigma 1.5 REVERSE, seed 1; host wall time per call (upload, filter, "
                     "download), median of 10 after 2 warm-up calls"}
    lib = kcv.lib()
    pinned_src = torch.from_numpy(host.copy()).pin_memory()
    pinned_dst = torch.empty_like(pinned_src).pin_memory()
    for threads in (1, cores):
        pool = kcv.ThreadPool(threads)
        for kind in ("pageable", "pinned"):
            if kind == "pageable":
                sp, dst = host.ctypes.data, np.zeros_like(host)
                dp = dst.ctypes.data
            else:
                sp, dp = pinned_src.data_ptr(), pinned_dst.data_ptr()
            times = []
            for i in range(12):
                t0 = _t.perf_counter()
                e = lib.kleidicv_gpu_thread_gaussian_blur_u8(sp, w * c, dp, w * c, w, h, c, 7, 7, 1.5, 1.5,
                                                             kcv.REVERSE, pool.mt)
                t1 = _t.perf_counter()
                assert e == kcv.OK, e
                if i >= 2:
                    times.append(t1 - t0)
            ms = 1e3 * float(np.median(times))
            out[f"{kind}_threads{threads}"] = {"ms_per_call": round(ms, 3),
                                               "mpix_s": round(w * h / (ms * 1e-3) / 1e6, 1)}
        pool.close()
    return out


def section_median(torch, kcv, ctx, stream):
    """Median blur, 1920x1080 (seed 6): u8 1 and 3 channels with K = 3, 5, 7
    (selection per element) and K = 15 (sliding histograms), f32 1 channel
    with K = 5; per-call time and bit-exactness on 16 rows against the
    oracle."""
    from oracle import oracle

    w, h = 1920, 1080
    rng = np.random.default_rng(6)
    out = {"config": "1920x1080, REPLICATE, seed 6; CUDA events over 20 calls"}
    for dtype, c, k in (("u8", 1, 3), ("u8", 1, 5), ("u8", 1, 7), ("u8", 3, 5), ("u8", 1, 15), ("f32", 1, 5)):
        dt = oracle.MEDIAN_DTYPES[dtype]
        host = rng.integers(0, 256, (h, w * c)).astype(dt)
        src = torch.from_numpy(host).cuda()
        dst = torch.empty_like(src)
        es = host.itemsize

        def call(i):
            e = kcv.median_blur(dtype, src.data_ptr(), w * c * es, dst.data_ptr(), w * c * es, w, h, c, k, k,
                                kcv.REPLICATE, ctx)
            assert e == kcv.OK, e

        call(0)
        ms = _events_time(torch, stream, call, 20)
        rows = list(range(0, h, h // 16))[:16]
        exact = bool(np.array_equal(dst.cpu().numpy()[rows],
                                    oracle.median_blur(host, w, h, c, k, kcv.REPLICATE, out_rows=rows)))
        out[f"{dtype}_c{c}_k{k}"] = {"us_per_call": round(ms * 1e3, 1),
                                     "mpix_s": round(w * h / (ms * 1e-3) / 1e6, 1), "bit_exact_rows": exact}
        del src, dst
    return out


def section_lk_pyramid(torch, kcv, ctx, stream):
    """kleidicv_gpu_build_optical_flow_pyr_lk_pyramid on 1920x1080x1, 4 levels,
    21x21 window (seed 7): device time per build + release (bordered images
    and Scharr pairs of every level, device memory from the context pool),
    and level 1 (image and Scharr interiors) against the oracle."""
    from oracle import oracle

    w, h, c, levels, win = 1920, 1080, 1, 4, 21
    rng = np.random.default_rng(7)
    host = _pyr_image(rng, w, h, c)
    src = torch.from_numpy(host).cuda()

    def build(i):
        pyr = kcv.LKPyramid(src.data_ptr(), w * c, w, h, c, levels, win, win, ctx)
        assert pyr.error == kcv.OK, pyr.error
        pyr.close()

    for i in range(3):
        build(i)
    ms = _events_time(torch, stream, build, 20)
    pyr = kcv.LKPyramid(src.data_ptr(), w * c, w, h, c, levels, win, win, ctx)
    torch.cuda.synchronize()
    lw, lh, img, istr, sch, sstr, bw, bh = pyr.level(1)
    got_img = torch.empty(lh * istr, dtype=torch.uint8, device="cuda")
    _copy_device(got_img.data_ptr(), img, (lh - 1) * istr + lw * c)
    got_sch = torch.empty(lh * sstr, dtype=torch.uint8, device="cuda")
    _copy_device(got_sch.data_ptr(), sch, (lh - 1) * sstr + lw * c * 4)
    gi = got_img.cpu().numpy().reshape(lh, istr)[:, : lw * c]
    gs = got_sch.cpu().numpy().reshape(lh, sstr)[:, : lw * c * 4].copy().view(np.int16)
    pyr.close()
    _, want = oracle.lk_pyramid(host, w, h, c, levels, win, win)
    lv = want[1]
    exact = bool(np.array_equal(gi, lv["image"][bh:bh + lh, bw * c:(bw + lw) * c]) and
                 np.array_equal(gs, lv["scharr"]))
    return {"config": "1920x1080x1, 4 levels, 21x21 window, seed 7; CUDA events over 20 build+release cycles",
            "ms_per_build": round(ms, 4), "mpix_s_level0": round(w * h / (ms * 1e-3) / 1e6, 1),
            "level1_bit_exact": exact}


def _log_uniform(rng, lo, hi):
    return int(round(float(np.exp(rng.uniform(np.log(lo), np.log(hi))))))


def section_batched(torch, kcv, ctx, stream, cores):
    """512 u8 images (seed 2): w 64-4096, h 64-2160 log-uniform, C in {1,3,4},
    Gaussian k in {3,5,7,15}, sigma 0.5-4, random border: one CUDA-graph
    launch of the batch plan against 512 plain calls and the CPU oracle."""
    from oracle import oracle

    rng = np.random.default_rng(2)
    items = []
    for _ in range(512):
        w, h = _log_uniform(rng, 64, 4096), _log_uniform(rng, 64, 2160)
        c = int(rng.choice([1, 3, 4]))
        k = int(rng.choice([3, 5, 7, 15]))
        sigma = float(rng.uniform(0.5, 4.0))
        border = int(rng.choice([kcv.REPLICATE, kcv.REFLECT, kcv.WRAP, kcv.REVERSE]))
        host = rng.integers(0, 256, (h, w * c), dtype=np.uint8)
        src = torch.from_numpy(host).cuda()
        dst = torch.empty_like(src)
        items.append((host, src, dst, w, h, c, k, sigma, border))
    mpix = sum(it[3] * it[4] for it in items) / 1e6
    nbytes = sum(2 * it[0].nbytes for it in items)
    reqs = [kcv.make_request(kcv.OP_GAUSSIAN_BLUR_U8, it[1].data_ptr(), it[3] * it[5], it[2].data_ptr(),
                             it[3] * it[5], it[3], it[4], it[5], it[6], it[6], it[7], it[7], border_type=it[8])
            for it in items]
    t0 = time.perf_counter()
    plan = kcv.BatchPlan(reqs, ctx)
    plan_ms = (time.perf_counter() - t0) * 1e3
    assert all(st == kcv.OK for st in plan.statuses), plan.statuses
    for _ in range(3):
        assert plan.launch(True) == kcv.OK
    graph_ms = _events_time(torch, stream, lambda i: plan.launch(True), 20)

    def plain(i):
        for it in items:
            e = kcv.gaussian_blur_u8(it[1].data_ptr(), it[3] * it[5], it[2].data_ptr(), it[3] * it[5], it[3],
                                     it[4], it[5], it[6], it[6], it[7], it[7], it[8], ctx)
            assert e == kcv.OK

    plain(0)
    plain_ms = _events_time(torch, stream, plain, 3)
    # Outputs of the batched launch against the oracle on a sample.
    plan.launch(True)
    torch.cuda.synchronize()
    exact = True
    for it in items[:8]:
        _, want = oracle.gaussian_blur_u8(it[0], it[3], it[4], it[5], it[6], it[7], it[8], nthreads=cores)
        exact &= bool(np.array_equal(it[2].cpu().numpy(), want))
    sample = items[:24]
    t0 = time.perf_counter()
    for it in sample:
        oracle.gaussian_blur_u8(it[0], it[3], it[4], it[5], it[6], it[7], it[8], nthreads=cores)
    cpu_s = time.perf_counter() - t0
    cpu_mpix = sum(it[3] * it[4] for it in sample) / 1e6
    tiles = plan.tile_count()
    plan.close()
    return {"config": "512 u8 images seed 2: w 64-4096, h 64-2160 log-uniform, C {1,3,4}, k {3,5,7,15}, "
                      "sigma 0.5-4, random border",
            "images": 512, "mpix": round(mpix, 1), "tiles": tiles,
            "graph_ms": round(graph_ms, 3), "graph_mpix_s": round(mpix / (graph_ms * 1e-3), 1),
            "graph_hbm_gbs": round(nbytes / (graph_ms * 1e-3) / 1e9, 1),
            "plain_calls_ms": round(plain_ms, 3), "plain_mpix_s": round(mpix / (plain_ms * 1e-3), 1),
            "speedup_vs_plain": round(plain_ms / graph_ms, 2), "plan_build_ms": round(plan_ms, 2),
            "cpu_oracle_mpix_s": round(cpu_mpix / cpu_s, 1), "cpu_sample": f"24 images, {cores} threads",
            "bit_exact_vs_oracle_sample": exact}


def _pyr_image(rng, w, h, c):
    y, x = np.mgrid[0:h, 0:w]
    base = 128 + 60 * np.sin(x / 17.0 + y / 29.0)
    img = np.repeat(base[:, :, None], c, axis=2) + rng.uniform(-40, 40, (h, w, c))
    return np.clip(np.rint(img), 0, 255).astype(np.uint8).reshape(h, w * c)


def section_pyramid(torch, kcv, ctx, stream):
    """Seed 3: 8192x8192x1 and 4096x4096x3 through 5 blur_and_downsample
    levels (REVERSE), each pyramid one launch; and 64 pyramids of 1024x768x4,
    5 levels each, in one launch.  Source and level buffers rotate over sets
    whose total exceeds twice the L2, so every call reads its level 0 from
    HBM.  Every level of the first set is compared with the CPU oracle."""
    from oracle import oracle

    rng = np.random.default_rng(3)
    l2 = 2 * 129 * 1024 * 1024
    out = {}

    def levels_of(w, h):
        sizes = []
        for _ in range(5):
            w, h = (w + 1) // 2, (h + 1) // 2
            sizes.append((w, h))
        return sizes

    def check(host, w, h, c, dsts):
        level, lw, lh = host, w, h
        for d in dsts:
            e, level = oracle.blur_and_downsample_u8(level, lw, lh, c, kcv.REVERSE, nthreads=os.cpu_count() or 1)
            lw, lh = (lw + 1) // 2, (lh + 1) // 2
            if e != 0 or not np.array_equal(d.cpu().numpy(), level):
                return False
        return True

    for (w, h, c) in ((8192, 8192, 1), (4096, 4096, 3)):
        host = _pyr_image(rng, w, h, c)
        sizes = levels_of(w, h)
        per_set = host.nbytes + sum(ww * hh * c for ww, hh in sizes)
        nsets = max(2, -(-l2 // per_set) + 1)
        sets = []
        for _ in range(nsets):
            src = torch.from_numpy(host).cuda()
            sets.append((src, [torch.empty((hh_, ww_ * c), dtype=torch.uint8, device="cuda") for ww_, hh_ in sizes]))

        def run(i, sets=sets, w=w, h=h, c=c):
            src, dsts = sets[i % len(sets)]
            e = kcv.build_pyramid_u8(src.data_ptr(), w * c, w, h, c, [d.data_ptr() for d in dsts],
                                     [d.stride(0) for d in dsts], kcv.REVERSE, ctx)
            assert e == kcv.OK

        for i in range(3):
            run(i)
        ms = _events_time(torch, stream, run, 20)
        torch.cuda.synchronize()
        out[f"{w}x{h}x{c}"] = {"ms": round(ms, 4), "mpix_s_level0": round(w * h / (ms * 1e-3) / 1e6, 1),
                               "hbm_gbs": round(per_set / (ms * 1e-3) / 1e9, 1), "launches_per_pyramid": 1,
                               "rotating_sets": nsets, "all_levels_bit_exact": check(host, w, h, c, sets[0][1])}
        del sets
    # 64 pyramids of 1024x768x4, 5 levels each: one launch.
    w, h, c = 1024, 768, 4
    sizes = levels_of(w, h)
    hosts = [_pyr_image(rng, w, h, c) for _ in range(64)]
    per_set = 64 * (w * h * c + sum(ww * hh * c for ww, hh in sizes))
    nsets = max(2, -(-l2 // per_set) + 1)
    bsets = []
    for _ in range(nsets):
        srcs = [torch.from_numpy(hh).cuda() for hh in hosts]
        dsts = [[torch.empty((lh, lw * c), dtype=torch.uint8, device="cuda") for lw, lh in sizes] for _ in srcs]
        bsets.append((srcs, dsts))

    # The call's arguments converted once per set (the timed loop makes only the C call).
    batches = [kcv.PyramidBatch([(s_.data_ptr(), w * c, w, h, c, [d.data_ptr() for d in ds],
                                  [d.stride(0) for d in ds], kcv.REVERSE) for s_, ds in zip(srcs, dsts)])
               for srcs, dsts in bsets]

    def run_b(i):
        err, _ = batches[i % len(batches)].launch(ctx)
        assert err == kcv.OK

    for i in range(3):
        run_b(i)
    ms = _events_time(torch, stream, run_b, 20)
    torch.cuda.synchronize()
    exact = all(check(hosts[k], w, h, c, bsets[0][1][k]) for k in (0, 31, 63))
    out["batched_64x1024x768x4"] = {"ms": round(ms, 4), "mpix_s_level0": round(64 * w * h / (ms * 1e-3) / 1e6, 1),
                                    "hbm_gbs": round(per_set / (ms * 1e-3) / 1e9, 1), "launches": 1,
                                    "rotating_sets": nsets, "all_levels_bit_exact_sample": exact}
    return out


def section_serving(torch, kcv, seconds, rate, high_seconds=10.0, inflight=3, batch_requests=512,
                    batch_mb=0):
    """Seed 4: Poisson arrivals at `rate` requests/s for `seconds`; 0.60
    gaussian_blur_u8 / 0.25 separable_filter_2d_u16 / 0.15
    blur_and_downsample_u8; w 320-7680, h 240-4320 log-uniform, C {1,3,4},
    Gaussian k {3,5,7,15}, separable 5x5, random border; images resident in the
    server's 40 GB pool.  Requests draw from 48 resident source images of those
    shapes, each with a ring of 16 output buffers (a buffer is reused 16
    requests of its image later, long after that request completed).  Every
    500th request of each run writes to a buffer of its own instead, and those
    outputs are compared byte for byte with the CPU oracle after the run."""
    from oracle import oracle

    rng = np.random.default_rng(4)
    srv = kcv.Server(0, pool_limit_bytes=40 << 30, max_inflight_batches=inflight, max_batch_requests=batch_requests,
                     max_batch_bytes=batch_mb << 20)
    templates = []
    for _ in range(48):
        u = rng.random()
        op = "gauss" if u < 0.60 else ("sep" if u < 0.85 else "bd")
        w, h = _log_uniform(rng, 320, 7680), _log_uniform(rng, 240, 4320)
        c = int(rng.choice([1, 3, 4]))
        dtype = np.uint16 if op == "sep" else np.uint8
        host = rng.integers(0, np.iinfo(dtype).max + 1, (h, w * c), dtype=dtype)
        ptr = srv.alloc(host.nbytes)
        assert ptr, "pool exhausted"
        staging = torch.from_numpy(host.view(np.uint8).reshape(-1)).cuda()
        _copy_device(ptr, staging.data_ptr(), host.nbytes)
        del staging
        tp = dict(op=op, w=w, h=h, c=c, dtype=dtype, src=ptr, next=0, host=host)
        ow, oh = ((w + 1) // 2, (h + 1) // 2) if op == "bd" else (w, h)
        tp["mpix"] = ow * oh / 1e6
        tp["out_bytes"] = ow * oh * c * np.dtype(dtype).itemsize
        tp["ring"] = [srv.alloc(tp["out_bytes"]) for _ in range(16)]
        assert all(tp["ring"]), "pool exhausted"
        templates.append(tp)
    torch.cuda.synchronize()

    def make_req(tp, dst=None):
        es = np.dtype(tp["dtype"]).itemsize
        if dst is None:
            dst = tp["ring"][tp["next"] % 16]
            tp["next"] += 1
        border = int(rng.choice([1, 2, 3, 4]))
        if tp["op"] == "gauss":
            k = int(rng.choice([3, 5, 7, 15]))
            sigma = float(rng.uniform(0.5, 4.0))
            return kcv.make_request(kcv.OP_GAUSSIAN_BLUR_U8, tp["src"], tp["w"] * tp["c"], dst, tp["w"] * tp["c"],
                                    tp["w"], tp["h"], tp["c"], k, k, sigma, sigma, border_type=border)
        if tp["op"] == "sep":
            return kcv.make_request(kcv.OP_SEPARABLE_U16, tp["src"], tp["w"] * tp["c"] * es, dst,
                                    tp["w"] * tp["c"] * es, tp["w"], tp["h"], tp["c"], 5, 5,
                                    kernel_x=list(rng.integers(0, 5, 5)), kernel_y=list(rng.integers(0, 5, 5)),
                                    border_type=border)
        ow = (tp["w"] + 1) // 2
        return kcv.make_request(kcv.OP_BLUR_AND_DOWNSAMPLE_U8, tp["src"], tp["w"] * tp["c"], dst, ow * tp["c"],
                                tp["w"], tp["h"], tp["c"], border_type=border)

    checked = []  # (template, request, own output buffer)
    cap = [30]    # checked requests per run

    def build(n, r):
        arrivals = np.cumsum(rng.exponential(1.0 / r, n))
        picks = rng.integers(0, len(templates), n)
        reqs = []
        for k, t in enumerate(picks):
            tp = templates[t]
            if k % 500 == 250 and len(checked) < cap[0]:
                own = srv.alloc(tp["out_bytes"])
                if own:
                    req = make_req(tp, own)
                    checked.append((tp, req, own))
                    reqs.append((tp, req))
                    continue
            reqs.append((tp, make_req(tp)))
        return arrivals, reqs

    def drive(arrivals, reqs):
        pending, lat, qlat, mpix, busy, failed = {}, [], [], 0.0, 0, 0
        n, i = len(reqs), 0
        t_start = time.perf_counter()
        while i < n or pending:
            now = time.perf_counter() - t_start
            while i < n and arrivals[i] <= now:
                err, rid = srv.submit(reqs[i][1])
                if err == kcv.OK:
                    pending[rid] = reqs[i][0]
                else:
                    busy += 1
                i += 1
            for rid, st, ta, tad, tc in srv.poll(256, timeout_ms=0):
                tp = pending.pop(rid)
                failed += st != kcv.OK
                lat.append((tc - ta) * 1e3)
                qlat.append((tad - ta) * 1e3)
                mpix += tp["mpix"]
            if i < n and not pending:
                time.sleep(max(0.0, min(arrivals[i] - (time.perf_counter() - t_start), 0.0005)))
        wall = time.perf_counter() - t_start
        lat, qlat = np.array(lat), np.array(qlat)
        return {"queue_p50_ms": round(float(np.percentile(qlat, 50)), 3),
                "queue_p99_ms": round(float(np.percentile(qlat, 99)), 3),
                "requests": n, "completed": int(len(lat)), "busy": busy, "failed": int(failed),
                "seconds": round(wall, 2), "offered_req_s": round(n / arrivals[-1], 1),
                "mpix_s": round(mpix / wall, 1),
                "p50_ms": round(float(np.percentile(lat, 50)), 3), "p99_ms": round(float(np.percentile(lat, 99)), 3),
                "p999_ms": round(float(np.percentile(lat, 99.9)), 3)}

    warm_arr, warm_reqs = build(200, rate)
    drive(warm_arr - warm_arr[0], warm_reqs)  # warm-up
    checked.clear()
    arrivals, reqs = build(int(seconds * rate), rate)
    n_main_checked = len(checked)
    main_run = drive(arrivals, reqs)
    srv.drain()
    # The first 1000 requests as plain per-request calls back to back and as one batch plan.
    ctx = kcv.Context.for_torch(0)
    stream = torch.cuda.current_stream()
    sample = reqs[:1000]
    sample_mpix = sum(tp["mpix"] for tp, _ in sample)

    def plain(_):
        for _tp, r in sample:
            e = _plain_call(kcv, r, ctx)
            assert e == kcv.OK, e

    plain(0)
    plain_ms = _events_time(torch, stream, plain, 1)
    plan = kcv.BatchPlan([r for _, r in sample], ctx)
    plan.launch(True)
    batch_ms = _events_time(torch, stream, lambda _: plan.launch(True), 3)
    plan.close()
    batched_mpix_s = sample_mpix / (batch_ms * 1e-3)
    # The plain calls and the batch above rewrote the checked outputs with the
    # same bytes; the comparison below covers the served results regardless.
    # Sustained load at 80% of the batched throughput.
    mean_mpix = float(np.mean([tp["mpix"] for tp, _ in reqs]))
    high_rate = 0.8 * batched_mpix_s / mean_mpix
    cap[0] = len(checked) + 30
    arr_h, reqs_h = build(int(high_seconds * high_rate), high_rate)
    high_run = drive(arr_h, reqs_h)
    srv.drain()
    ctx.close()
    # Served outputs against the CPU oracle, byte for byte.
    exact, n_checked = True, 0
    for tp, r, own in checked:
        got = np.empty(tp["out_bytes"], np.uint8)
        _copy_to_host(got, own)
        if tp["op"] == "gauss":
            e, want = oracle.gaussian_blur_u8(tp["host"], tp["w"], tp["h"], tp["c"], r.kernel_width, r.sigma_x,
                                              r.border_type, nthreads=os.cpu_count() or 1)
        elif tp["op"] == "sep":
            e, want = oracle.separable_filter_2d(tp["host"], tp["w"], tp["h"], tp["c"],
                                                 np.array(list(r.kernel_x)[:5], np.uint16),
                                                 np.array(list(r.kernel_y)[:5], np.uint16), r.border_type,
                                                 nthreads=os.cpu_count() or 1)
        else:
            e, want = oracle.blur_and_downsample_u8(tp["host"], tp["w"], tp["h"], tp["c"], r.border_type,
                                                    nthreads=os.cpu_count() or 1)
        exact &= e == 0 and np.array_equal(got, np.ascontiguousarray(want).view(np.uint8).reshape(-1))
        n_checked += 1
    srv.close()
    out = {"config": f"Poisson {rate:.0f} req/s for {seconds:.1f} s (seed 4), mix 0.60/0.25/0.15, "
                     "w 320-7680 h 240-4320 log-uniform, 48 resident source images, 40 GB pool, "
                     f"{inflight} batches in flight, <= {batch_requests} requests"
                     + (f" and <= {batch_mb} MiB of image traffic" if batch_mb else "") + " per batch"}
    out.update(main_run)
    out.update({"plain_per_request_mpix_s": round(sample_mpix / (plain_ms * 1e-3), 1),
                "batched_mpix_s": round(batched_mpix_s, 1), "comparison_sample": f"first {len(sample)} requests",
                "load_80pct_of_batched": high_run,
                "served_bit_exact": bool(exact), "served_checked": n_checked,
                "served_check": f"every 500th request of each run (at most 30 per run; {n_main_checked} in the "
                                "configured run), own output buffer, against the CPU oracle"})
    return out


def _copy_to_host(host_array, src_ptr):
    """Device bytes at a raw pointer -> a host numpy array (cudaMemcpy through ctypes)."""
    import ctypes

    lib = _cudart()
    lib.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    err = lib.cudaMemcpy(ctypes.c_void_p(host_array.ctypes.data), ctypes.c_void_p(src_ptr),
                         ctypes.c_size_t(host_array.nbytes), 2)
    assert err == 0, err


def _with_dst(kcv, r, dst):
    return kcv.make_request(r.op, r.src, r.src_stride, dst, r.dst_stride, r.width, r.height, r.channels,
                            r.kernel_width, r.kernel_height, r.sigma_x, r.sigma_y, list(r.kernel_x),
                            list(r.kernel_y), r.border_type, r.border_value, r.allow_extensions)


def _plain_call(kcv, r, ctx):
    if r.op == kcv.OP_GAUSSIAN_BLUR_U8:
        return kcv.gaussian_blur_u8(r.src, r.src_stride, r.dst, r.dst_stride, r.width, r.height, r.channels,
                                    r.kernel_width, r.kernel_height, r.sigma_x, r.sigma_y, r.border_type, ctx)
    if r.op == kcv.OP_SEPARABLE_U16:
        return kcv.separable_filter_2d("u16", r.src, r.src_stride, r.dst, r.dst_stride, r.width, r.height,
                                       r.channels, list(r.kernel_x), 5, list(r.kernel_y), 5, r.border_type, ctx)
    return kcv.blur_and_downsample_u8(r.src, r.src_stride, r.width, r.height, r.dst, r.dst_stride, r.channels,
                                      r.border_type, ctx)


def _copy_device(dst_ptr, src_ptr, nbytes):
    """Device-to-device copy between raw pointers (cudaMemcpy through ctypes)."""
    import ctypes

    lib = _cudart()
    lib.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    err = lib.cudaMemcpy(ctypes.c_void_p(dst_ptr), ctypes.c_void_p(src_ptr), ctypes.c_size_t(nbytes), 3)
    assert err == 0, err


_CUDART = None


def _cudart():
    import ctypes
    import glob

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
    return _CUDART


def run_sections(args, names):
    import torch
    import __graft_entry__ as ge

    kcv = ge.package()
    stream = torch.cuda.current_stream()
    ctx = kcv.Context(torch.cuda.current_device(), stream.cuda_stream)
    cores = os.cpu_count() or 1
    out = {}
    for name in names:
        t0 = time.perf_counter()
        try:
            if name == "c1":
                out[name] = section_c1(torch, kcv, ctx, stream)
            elif name == "batched":
                out[name] = section_batched(torch, kcv, ctx, stream, cores)
            elif name == "pyramid":
                out[name] = section_pyramid(torch, kcv, ctx, stream)
            elif name == "lk_pyramid":
                out[name] = section_lk_pyramid(torch, kcv, ctx, stream)
            elif name == "median":
                out[name] = section_median(torch, kcv, ctx, stream)
            elif name == "thread_api":
                out[name] = section_thread_api(torch, kcv, cores)
            elif name == "sobel":
                out[name] = section_sobel(torch, kcv, ctx, stream, cores)
            elif name == "serving":
                out[name] = section_serving(torch, kcv, args.serving_seconds, args.serving_rate,
                                            args.serving_high_seconds, args.serving_inflight,
                                            batch_mb=args.serving_batch_mb)
        except Exception as e:  # a failed section must not lose the headline line
            out[name] = {"error": f"{type(e).__name__}: {e}"}
        out[name]["section_seconds"] = round(time.perf_counter() - t0, 1)
        torch.cuda.empty_cache()
    ctx.close()
    return out


# ----------------------------------------------------------------------------

def reference_arm(args, calls, config):
    """`--impl reference`: the reference's own CPU path (kleidicv_thread_* on all
    host cores) on this workload, K timed steps after W warm-up steps.  One full
    pass calibrates the step: when K full passes would take more than
    REF_BUDGET_S, every step filters the same top band of rows of each image
    instead (a bounded sample; the rate counts the sampled pixels).  Where the
    reference cannot be loaded (not an AArch64 host, or its build failed), the
    CPU restatement of its algorithm stands in, and the line says why."""
    cores = os.cpu_count() or 1
    ref, info = reference_cpu()
    if ref is not None:
        plan = ref_plan(calls)
        pool = ref.Pool(cores)
        run = lambda rows: ref_pass(plan, pool, rows=rows)  # noqa: E731
        kind = "reference"
        what = (f"kleidicv_thread_* on a persistent std::thread pool of {cores} threads (KleidiCV built from "
                f"its sources on this host, default dispatch); " + REF_STANDIN)
    else:
        from oracle import oracle

        oracle.build()
        pool = None
        run = lambda rows: cpu_pass(calls, cores, rows=rows)  # noqa: E731
        kind = "port"
        what = f"CPU restatement oracle/kcv_oracle.c on {cores} threads; the reference is not available: {info}"
    try:
        t0 = time.perf_counter()
        run(H)
        full_s = time.perf_counter() - t0
        rows = H
        if args.steps * full_s > REF_BUDGET_S:
            rows = max(64, int(H * REF_BUDGET_S / (args.steps * full_s)))
        for _ in range(args.warmup):
            run(rows)
        times = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            run(rows)
            times.append(time.perf_counter() - t0)
    finally:
        if pool is not None:
            pool.close()
    ms = 1e3 * sum(times) / len(times)
    mpix = len(calls) * W * rows / 1e6
    v = round(mpix / (ms / 1e3), 2)
    cb = {"value": v, "unit": METRIC, "cores": cores, "kind": kind,
          "sample": f"each step one pass of 7 calls over rows 0..{rows - 1} of each {W}x{H} image (a full "
                    f"pass: {1e3 * full_s:.0f} ms); {what}"}
    if ref is not None:
        cb["host"] = info
    return {"metric": METRIC, "value": v, "unit": METRIC, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8/u16", "data": "synthetic",
            "config": config, "impl": "reference", "cpu_baseline": cb,
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def profile_op(name, range_calls=0):
    """One workload for a profiler capture (`--profile-op`): three calls, or
    with range_calls > 0 one call, then range_calls calls over rotating buffer
    sets (more than twice the L2 in total) inside a profiler range."""
    import torch
    import __graft_entry__ as ge

    kcv = ge.package()
    ctx = kcv.Context.for_torch(0)
    calls, _ = make_calls()
    rng = np.random.default_rng(3)
    if name in ("gauss", "u16", "s16"):
        c = {"gauss": calls[0], "u16": calls[1], "s16": calls[4]}[name]
        host = c["src"].view(np.uint8)
        out_shape, out_dtype = host.shape, torch.uint8
    elif name == "blurdown":
        host = _pyr_image(rng, 4096, 4096, 1)
        out_shape, out_dtype = (2048, 2048), torch.uint8
    elif name == "arbitrary":
        host = rng.integers(0, 256, (H, W), dtype=np.uint8)
        out_shape, out_dtype = (H, W), torch.uint8
    elif name in ("median5", "median15", "lk"):
        host = rng.integers(0, 256, (1080, 1920), dtype=np.uint8)
        out_shape, out_dtype = (1080, 1920), torch.uint8
    else:
        host = rng.integers(0, 256, (H, W), dtype=np.uint8)
        out_shape, out_dtype = (H, W), torch.int16
    nbytes = 2 * host.nbytes
    nsets = max(1, -(-2 * 129 * 1024 * 1024 // nbytes) + 1) if range_calls else 1
    sets = [(torch.from_numpy(host).cuda(), torch.empty(out_shape, dtype=out_dtype, device="cuda"))
            for _ in range(nsets)]

    def f(i):
        src, dst = sets[i % nsets]
        ss = src.stride(0)
        if name == "gauss":
            return kcv.gaussian_blur_u8(src.data_ptr(), ss, dst.data_ptr(), ss, W, H, 4, 7, 7, 1.5, 1.5,
                                        c["border"], ctx)
        if name in ("u16", "s16"):
            return kcv.separable_filter_2d(c["dtype"], src.data_ptr(), ss, dst.data_ptr(), ss, W, H, 1, c["kx"], 5,
                                           c["ky"], 5, c["border"], ctx, border_value=c["bv"])
        if name == "blurdown":
            return kcv.blur_and_downsample_u8(src.data_ptr(), 4096, 4096, 4096, dst.data_ptr(), 2048, 1,
                                              kcv.REVERSE, ctx)
        if name == "arbitrary":
            return kcv.gaussian_blur_u8(src.data_ptr(), W, dst.data_ptr(), W, W, H, 1, 31, 31, 5.0, 5.0,
                                        kcv.REPLICATE, ctx)
        if name in ("median5", "median15"):
            k = 5 if name == "median5" else 15
            return kcv.median_blur("u8", src.data_ptr(), 1920, dst.data_ptr(), 1920, 1920, 1080, 1, k, k,
                                   kcv.REPLICATE, ctx)
        if name == "lk":
            pyr = kcv.LKPyramid(src.data_ptr(), 1920, 1920, 1080, 1, 4, 21, 21, ctx)
            err = pyr.error
            if err == kcv.OK:
                pyr.close()
            return err
        return kcv.sobel_3x3_horizontal_s16_u8(src.data_ptr(), W, dst.data_ptr(), 2 * W, W, H, 1, ctx)

    n = 3 if not range_calls else 1
    for i in range(n):
        if f(i) != kcv.OK:
            raise RuntimeError(f"{name} call failed")
    if range_calls:
        torch.cuda.synchronize()
        torch.cuda.profiler.start()
        for i in range(range_calls):
            if f(1 + i) != kcv.OK:
                raise RuntimeError(f"{name} call failed")
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
    if ctx.synchronize() != kcv.OK:
        raise RuntimeError(f"{name} failed on the device")
    ctx.close()
    print(f"profile-op {name}: done ({n} + {range_calls} calls, {nsets} buffer sets)", flush=True)


def main():
    args = parse_args()
    if args.profile_op:
        profile_op(args.profile_op, args.profile_range)
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    calls, taps = make_calls()
    mpix = out_pixels(calls) / 1e6
    config = {"workload": WORKLOAD, "calls_per_step": len(calls), "images": f"{W}x{H}",
              "taps": taps, "seed": 1,
              "l2": f"{N_SETS} rotating buffer sets of {N_SETS * algorithmic_bytes(calls) / 1e6:.0f} MB "
                    f"total (> 4x the 129 MB L2)",
              "parallelism": f"replicas x{world}"}

    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(reference_arm(args, calls, config)), flush=True)
        return

    if world > 1:
        import torch

        torch.distributed.init_process_group("nccl")
    res, close = run_gpu(args, rank, world, calls, taps)
    peak, peak_kind = measured_hbm_peak()
    g_ms = res["per_call"][0]
    achieved = GAUSS_BYTES / (g_ms * 1e-3) / 1e9
    line = {
        "metric": METRIC,
        "value": round(whole_job_rate(mpix, world, res["ms_step"]), 1),
        "unit": METRIC,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(res["ms_step"], 5),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u8/u16/s16",
        "data": "synthetic",
        "config": config,
        "hbm_gbs": round(world * algorithmic_bytes(calls) / (res["ms_step"] * 1e-3) / 1e9, 1),
        "per_call_us": {c["name"]: round(1e3 * t, 2) for c, t in zip(calls, res["per_call"])},
        "per_call_note": "the Gaussian timed inside the timed region (every 8th step); the others each timed "
                         "alone afterwards",
        "roofline": {"kernel": "gauss8_kernel<7> (gaussian_blur_u8 3840x2160x4 7x7)",
                     "bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "peak_source": f"{peak_kind} hbm_gbs (copy bandwidth)",
                     "algorithmic_bytes_per_launch": GAUSS_BYTES,
                     "traffic": profiled_traffic(),
                     "back_to_back_us": round(res["gauss_b2b_ms"] * 1e3, 2),
                     "frac_back_to_back": round(GAUSS_BYTES / (res["gauss_b2b_ms"] * 1e-3) / 1e9 / peak, 4),
                     "note": f"achieved/frac: CUDA events around the launch on every {ROOFLINE_EVERY}th step "
                             "inside the timed region (launch ramp included); back_to_back: 100 launches "
                             "between two events"},
        "gpu_launches": res["launches"],
        "e2e": {"value": round(whole_job_rate(mpix, world, res["e2e_ms"]), 1), "unit": METRIC,
                "h2d_bytes_per_step": res["h2d"], "d2h_bytes_per_step": res["d2h"],
                "ms_per_step": round(res["e2e_ms"], 4)},
        "clocks": res["clocks"],
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb, exact = cpu_baseline(calls, args.cpu_passes, res["outputs"])
        line["cpu_baseline"] = cb
        line["bit_exact_vs_" + ("reference" if cb["kind"] == "reference" else "oracle")] = exact
    close()
    if rank == 0 and world == 1 and args.sections != "none":
        names = [n for n in args.sections.split(",") if n]
        line.update(run_sections(args, names))
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
