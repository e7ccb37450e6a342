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
measured HBM copy bandwidth; `cpu_baseline` is the CPU restatement of the
reference algorithm (oracle/kcv_oracle.c, all host cores) on the same inputs,
whose output is also compared byte for byte with the GPU's.

`--impl reference` times that CPU path alone (the reference itself is
AArch64 NEON/SVE C++ that cannot be built from its sources on either machine),
with all host threads, on the same workload.

Multi-GPU: images are independent, so N ranks run N replicas of the sweep with
no collective on the data path ("replicas only"); the step time is the max over
ranks and `value` counts the pixels of all ranks.
"""
from __future__ import annotations

import argparse
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
    p = os.path.join(REPO, "profiles", "sepfused_gauss7_rgba_4k.md")
    try:
        with open(p) as f:
            for line in f:
                if line.startswith("traffic_bytes_per_launch:"):
                    return int(line.split(":", 1)[1].strip())
    except (OSError, ValueError):
        pass
    return None


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

    def step(i, evs=None):
        for ci, (c, (src, dst)) in enumerate(zip(calls, sets[i % N_SETS])):
            if evs is not None:
                evs[ci][0].record(stream)
            issue(c, src.data_ptr(), src.stride(0) * src.element_size(), dst.data_ptr(),
                  dst.stride(0) * dst.element_size())
            if evs is not None:
                evs[ci][1].record(stream)

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
    for i in range(args.steps):
        step(i, ev_calls[i])
    t_end.record(stream)
    torch.cuda.synchronize()
    wall1 = time.time()
    barrier()
    launches = ctx.launch_count() - launches0
    sampler.stop()
    if ctx.synchronize() != kcv.OK:
        raise RuntimeError("timed region failed")
    for i in range(args.steps):
        for ci in range(len(calls)):
            per_call[ci].append(ev_calls[i][ci][0].elapsed_time(ev_calls[i][ci][1]))
    ms_total = t_begin.elapsed_time(t_end)
    if world > 1:
        t = torch.tensor([ms_total], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_total = float(t.item())
    ms_step = ms_total / args.steps

    # ---- end to end through the public calls with pinned host buffers.
    hsrc = [torch.from_numpy(c["src"].view(np.int16) if c["src"].dtype == np.uint16 else c["src"])
            .pin_memory() for c in calls]
    hdst = [torch.empty_like(h).pin_memory() for h in hsrc]
    dset = sets[0]
    h2d = sum(h.numel() * h.element_size() for h in hsrc)
    d2h = sum(h.numel() * h.element_size() for h in hdst)

    def e2e_step():
        for c, hs, hd, (src, dst) in zip(calls, hsrc, hdst, dset):
            src.copy_(hs, non_blocking=True)
            issue(c, src.data_ptr(), src.stride(0) * src.element_size(), dst.data_ptr(),
                  dst.stride(0) * dst.element_size())
            hd.copy_(dst, non_blocking=True)

    e2e_n = max(1, min(args.e2e_steps, args.steps))
    for _ in range(3):
        e2e_step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(e2e_n):
        e2e_step()
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / e2e_n
    if world > 1:
        t = torch.tensor([e2e_ms], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_ms = float(t.item())
    if ctx.synchronize() != kcv.OK:
        raise RuntimeError("end-to-end run failed")

    result = dict(ms_step=ms_step, per_call=[statistics.mean(v) for v in per_call],
                  launches=launches, e2e_ms=e2e_ms, h2d=h2d, d2h=d2h,
                  clocks=sampler.summary(wall0, wall1),
                  outputs=[hd.numpy() for hd in hdst] if rank == 0 else None)
    return result, (lambda: (ctx.close()))


# ----------------------------------------------------------------------------
# CPU restatement (oracle port, all host cores)
# ----------------------------------------------------------------------------

def cpu_pass(calls, nthreads, keep=False):
    from oracle import oracle

    outs = []
    for c in calls:
        if c["op"] == "gauss":
            err, out = oracle.gaussian_blur_u8(c["src"], W, H, c["channels"], c["ksize"], c["sigma"],
                                               c["border"], nthreads=nthreads)
        else:
            ext = c["bv"] is not None
            err, out = oracle.separable_filter_2d(c["src"], W, H, c["channels"], np.array(c["kx"]),
                                                  np.array(c["ky"]), c["border"], ext=ext,
                                                  border_value=c["bv"] or 0, nthreads=nthreads)
        if err != oracle.OK:
            raise RuntimeError(f"oracle {c['name']}: error {err}")
        if keep:
            outs.append(out)
    return outs


def cpu_baseline(calls, passes, outputs=None):
    from oracle import oracle

    oracle.build()
    cores = os.cpu_count() or 1
    outs = cpu_pass(calls, cores, keep=True)  # also warms the pages
    exact = None
    if outputs is not None:
        exact = all(np.array_equal(a.view(np.uint8), b.view(np.uint8)) for a, b in zip(outs, outputs))
    times = []
    for _ in range(passes):
        t0 = time.perf_counter()
        cpu_pass(calls, cores)
        times.append(time.perf_counter() - t0)
    sec = statistics.median(times)
    return dict(value=round(out_pixels(calls) / sec / 1e6, 2), unit=METRIC, cores=cores, kind="port",
                sample=f"{passes} full passes of the 7-call sweep (median) with {cores} threads; "
                       f"CPU restatement oracle/kcv_oracle.c (scalar C, -O3)"), exact


# ----------------------------------------------------------------------------

def main():
    args = parse_args()
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
        from oracle import oracle

        oracle.build()
        cores = os.cpu_count() or 1
        for _ in range(args.warmup):
            cpu_pass(calls[:1], cores)
        times = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            cpu_pass(calls, cores)
            times.append(time.perf_counter() - t0)
        ms = 1e3 * sum(times) / len(times)
        v = round(mpix / (ms / 1e3), 2)
        line = {"metric": METRIC, "value": v, "unit": METRIC, "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "u8/u16/s16", "data": "synthetic",
                "config": config, "impl": "reference",
                "cpu_baseline": {"value": v, "unit": METRIC, "cores": cores, "kind": "port",
                                 "sample": f"each step one full pass of the 7-call sweep on {cores} "
                                           "threads; CPU restatement of the reference algorithm "
                                           "(KleidiCV itself is AArch64 NEON/SVE C++ that cannot be "
                                           "built from its sources here)"},
                "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
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
        "value": round(world * mpix / (res["ms_step"] * 1e-3), 1),
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
        "roofline": {"kernel": "sepfused_kernel<SIGMA, 7, 4> (gaussian_blur_u8 3840x2160x4 7x7)",
                     "bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "peak_source": f"{peak_kind} hbm_gbs (copy bandwidth)",
                     "algorithmic_bytes_per_launch": GAUSS_BYTES,
                     "traffic": profiled_traffic()},
        "gpu_launches": res["launches"],
        "e2e": {"value": round(world * mpix / (res["e2e_ms"] * 1e-3), 1), "unit": METRIC,
                "h2d_bytes_per_step": res["h2d"], "d2h_bytes_per_step": res["d2h"],
                "ms_per_step": round(res["e2e_ms"], 4)},
        "clocks": res["clocks"],
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb, exact = cpu_baseline(calls, args.cpu_passes, res["outputs"])
        line["cpu_baseline"] = cb
        line["bit_exact_vs_oracle"] = exact
    if rank == 0:
        print(json.dumps(line), flush=True)
    close()
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
