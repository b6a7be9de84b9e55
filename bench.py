#!/usr/bin/env python3
"""Benchmark of the GB300 lifting hot path.

Workload (one GPU): a 16384 x 16384 float32 image (1 GiB, seeded smooth field
plus noise, integers in [0, 255]) under CDF 9/7, forward then inverse to the
full depth of 14 levels.  One step = that forward + inverse pair, so one step
processes 2 * 16384^2 pixels.

Printed JSON line (rank 0):
  value      Mpx/s of the step with the image resident in HBM (device API,
             out of place, CUDA events on the launching stream);
  e2e        the same metric through the drop-in C ABI (dwt_cdf97_2f_s /
             dwt_cdf97_2i_s) on a pinned host image: every step copies the
             image to the device and the coefficients / reconstruction back
             (extras.e2e_pageable_16384_mpx_s: the same on a pageable,
             malloc'ed image, as the reference's callers allocate it);
  roofline   the dominant kernel (level 0 of the forward transform) timed
             alone: algorithmic bytes (read + write, 8 B per pixel) over its
             average duration, against the measured HBM copy peak;
  cpu_baseline  the CPU restatement of the reference (OpenMP, all host
             cores) on the same image;
  errors_vs_fp64  per configuration, max and RMS error of the GPU output
             against the FP64 restatement (libdwt's double variants):
             forward relative to the FP64 coefficients' range, round trip
             to the input range (computed in the CPU leg, after the GPU work).
The inputs (1 GiB) are larger than L2 (129 MB), so no flush between steps.

--impl reference times the reference algorithm on the host cores (the
oracle's C restatement, since the reference library itself is compiled only
where its source is present) and prints the same line with impl=reference.

Multi-GPU: the path does not shard (one image per GPU); N GPUs run N
independent replicas and `value` is the pixels of all ranks over the slowest
rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W = H = 16384
J = 14
WORKLOAD = "cdf97 2D forward+inverse, 16384x16384 float32, j_max=14"


def hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks + throttle reasons every 100 ms in the background."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append((time.time(), [x.strip() for x in line.split(",")]))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self, t0: float, t1: float):
        win = [s for (t, s) in self.samples if t0 - 0.15 <= t <= t1 + 0.15]
        if not win:
            win = [s for (_, s) in self.samples]
        if not win:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        mhz = [float(s[1]) for s in win if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in win if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in win for i in range(4) if len(s) > 5 + i and s[5 + i] == "Active"})
        return {"sm_mhz": float(np.median(mhz)) if mhz else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(win)}


def cpu_baseline(img: np.ndarray, threads: int, min_s: float = 10.0, max_s: float = 30.0):
    """Time the oracle (C restatement of the reference, OpenMP on `threads`
    cores) on the workload: forward + inverse CDF 9/7 of the image, repeated
    until at least `min_s` seconds of CPU work; a band of full-width rows is
    used instead of the whole image only if one pair would exceed `max_s`."""
    from oracle import oracle as O
    probe = np.ascontiguousarray(img[:512])
    t = time.perf_counter()
    f, j = O.transform2_dense(probe, "cdf97", "f", -1, 0, "s", threads)
    O.transform2_dense(f, "cdf97", "i", j, 0, "s", threads)
    per_px = (time.perf_counter() - t) / (2 * probe.size)
    rows = img.shape[0]
    if per_px * 2 * img.size > max_s:
        rows = max(512, int(max_s / (per_px * 2 * img.shape[1])))
    sample = np.ascontiguousarray(img[:rows])
    pairs, t0 = 0, time.perf_counter()
    while True:
        f, j = O.transform2_dense(sample, "cdf97", "f", -1, 0, "s", threads)
        O.transform2_dense(f, "cdf97", "i", j, 0, "s", threads)
        pairs += 1
        if time.perf_counter() - t0 >= min_s:
            break
    dt = time.perf_counter() - t0
    mpx = pairs * 2 * sample.size / dt / 1e6
    return mpx, (f"{sample.shape[1]}x{sample.shape[0]} cdf97 forward+inverse full depth, "
                 f"{pairs} pairs in {dt:.1f} s")


def cpu_configs(threads: int, loops: int = 3) -> dict:
    """The CPU restatement's rate on every 2D configuration of the benchmark
    (forward + inverse, best of `loops` as the reference's perf harness
    measures, src/libdwt.c:8440-8492): the 1024^2 plain drop-in (j = 5) with
    each wavelet, the 16384^2 image with CDF 5/3, and the 16383 x 16385 odd
    size with each wavelet; Mpx/s of inner pixels per transform."""
    from libdwt_gb300 import synth
    from oracle import oracle as O
    out = {"cores": threads, "kind": "port", "unit": "Mpx/s (forward + inverse pair)", "loops": loops}
    cases = [("c0_1024_cdf97_j5", 1024, 1024, "cdf97", 5), ("c0_1024_cdf53_j5", 1024, 1024, "cdf53", 5),
             ("c1_16384_cdf53_j14", 16384, 16384, "cdf53", 14),
             ("c1_16383x16385_cdf97_j14", 16383, 16385, "cdf97", 14),
             ("c1_16383x16385_cdf53_j14", 16383, 16385, "cdf53", 14)]
    for name, w, h, wav, j in cases:
        img = synth_image() if (w, h) == (W, H) else synth.image(w, h, seed=0 if w == h else 1)
        best = float("inf")
        for _ in range(loops if w * h < 1 << 26 else 1):
            t = time.perf_counter()
            f, jj = O.transform2_dense(img, wav, "f", j, 0, "s", threads)
            O.transform2_dense(f, wav, "i", jj, 0, "s", threads)
            best = min(best, time.perf_counter() - t)
        out[name] = round(2 * w * h / best / 1e6, 1)
    return out


def cpu_checks(threads: int, main_img, main_coef, main_rec, checks: dict) -> dict:
    """The checker half of the CPU leg: max and RMS error of every
    configuration's GPU output against the oracle's FP64 transform (the
    restatement of libdwt's double variants), plus the bit-exact check of the
    signal banks against the float restatement.  Forward errors are relative
    to the range of the FP64 coefficients (deep coefficients grow by the
    scaling factor per level, so the float path's error grows with them),
    round-trip errors to the input's range.  The GPU outputs were produced
    before, without the oracle."""
    from oracle import oracle as O

    def rel(a, b):
        rng = float(b.max() - b.min()) or 1.0
        d = np.abs(a.astype(np.float64) - b)
        return {"max_rel": float(d.max() / rng), "rms_rel": float(np.sqrt((d ** 2).mean()) / rng)}

    out = {"normalisation": "forward: range of the FP64 coefficients; round trip: input range"}
    ref, _ = O.transform2_dense(main_img, "cdf97", "f", J, 0, "d", threads)
    out["c1_cdf97_fwd"] = rel(main_coef, ref)
    del ref
    out["c1_cdf97_roundtrip"] = rel(main_rec, main_img.astype(np.float64))
    if "c0" in checks:
        img0, coef0 = checks["c0"]
        ref0, j0 = O.transform2_dense(img0, "cdf97", "f", 5, 0, "d", threads)
        out["c0_cdf97_fwd_j5"] = rel(coef0, ref0)
    if "c2" in checks:
        worst = {"max_rel": 0.0, "rms_rel": 0.0}
        worst_rt = {"max_rel": 0.0, "rms_rel": 0.0}
        for img2, out2, wav, jj, back2 in checks["c2"]:
            ref2, _ = O.transform2_dense(img2, wav, "f", jj, 0, "d", threads)
            e = rel(out2, ref2)
            worst = {k: max(worst[k], e[k]) for k in worst}
            e = rel(back2, img2.astype(np.float64))
            worst_rt = {k: max(worst_rt[k], e[k]) for k in worst_rt}
        out["c2_sample_fwd_worst"] = dict(worst, images=len(checks["c2"]))
        out["c2_sample_roundtrip_worst"] = dict(worst_rt, images=len(checks["c2"]))
    if "c4" in checks:
        part, gpu_part, n, st, count, lanes, gs = checks["c4"]
        ref4 = part.copy()
        O.batch_1d_cdf97(ref4, n, st, count, lanes, gs, 4, False, threads)
        out["c4_fwd_bit_exact_vs_float_restatement"] = bool(np.array_equal(gpu_part, ref4))
        # the CPU baseline of C4: the float restatement over the same bank
        # layout (OpenMP over signals), forward, on a slice of 1024 groups
        bank = np.repeat(part, 16, axis=0)
        t0 = time.perf_counter()
        O.batch_1d_cdf97(bank, n, st, bank.shape[0] * lanes, lanes, gs, 4, False, threads)
        dt = time.perf_counter() - t0
        t0 = time.perf_counter()
        O.batch_1d_cdf97(bank, n, st, bank.shape[0] * lanes, lanes, gs, 4, True, threads)
        dti = time.perf_counter() - t0
        out["c4_cpu_fwd_gsamples_s"] = {"value": round(bank.size / dt / 1e9, 3), "cores": threads, "kind": "port",
                                        "sample": f"{bank.shape[0] * lanes} signals of {n}"}
        out["c4_cpu_inv_gsamples_s"] = {"value": round(bank.size / dti / 1e9, 3), "cores": threads, "kind": "port",
                                        "sample": f"{bank.shape[0] * lanes} signals of {n}"}
    return out


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("BENCH_BACKEND") != "gloo" else "gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(ws, x: float) -> float:
    """Max over ranks (the slowest rank's time)."""
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(ws: int, steps: int, px_step: int, ms_max: float) -> float:
    """Whole-job Mpx/s of N independent replicas: every rank's pixels over the
    slowest rank's time."""
    return ws * steps * px_step / (ms_max / 1e3) / 1e6


def run_reference(args, ws, rank):
    if rank != 0:
        return
    from oracle import oracle as O
    threads = O.max_threads()
    img = synth_image()
    # one step = forward + inverse on a band of full-width rows, sized so the
    # whole run stays within about two minutes
    from oracle import oracle as O2
    strip = np.ascontiguousarray(img[:256])
    t = time.perf_counter()
    f, j = O2.transform2_dense(strip, "cdf97", "f", -1, 0, "s", threads)
    O2.transform2_dense(f, "cdf97", "i", j, 0, "s", threads)
    per_px = (time.perf_counter() - t) / (2 * strip.size)
    budget = 120.0 / max(1, args.steps + args.warmup)
    rows = int(min(H, max(256, budget / (per_px * 2 * W))))
    sample = np.ascontiguousarray(img[:rows])
    for _ in range(args.warmup):
        f, j = O2.transform2_dense(sample, "cdf97", "f", -1, 0, "s", threads)
        O2.transform2_dense(f, "cdf97", "i", j, 0, "s", threads)
    t = time.perf_counter()
    for _ in range(args.steps):
        f, j = O2.transform2_dense(sample, "cdf97", "f", -1, 0, "s", threads)
        O2.transform2_dense(f, "cdf97", "i", j, 0, "s", threads)
    dt = time.perf_counter() - t
    mpx = args.steps * 2 * sample.size / dt / 1e6
    desc = f"{W}x{rows} rows of the workload image, cdf97 forward+inverse full depth per step"
    line = {"impl": "reference", "metric": "2D DWT throughput (CDF 9/7 forward+inverse, full depth)",
            "value": round(mpx, 3), "unit": "Mpx/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded blob field + noise, integers 0..255)",
            "config": {"workload": WORKLOAD, "sample": desc, "l2": "inputs larger than L2"},
            "cpu_baseline": {"value": round(mpx, 3), "unit": "Mpx/s", "cores": threads, "kind": "port",
                             "sample": desc},
            "e2e": {"value": round(mpx, 3), "unit": "Mpx/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


_IMG = None


def synth_image():
    global _IMG
    if _IMG is None:
        from libdwt_gb300 import synth
        _IMG = synth.image(W, H, seed=0)
    return _IMG


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--level-reps", type=int, default=50)
    ap.add_argument("--serve-seconds", type=float, default=10.0,
                    help="length of the serving replay in the extras")
    ap.add_argument("--image", type=int, default=16384,
                    help="image side (a smaller case for profiler captures)")
    ap.add_argument("--dropin-reps", type=int, default=10, help="timed pairs of each drop-in extra")
    ap.add_argument("--only", choices=["c2", "c3", "c4", "dropin", "dropin-dense", "sparse"], default=None,
                    help="run one secondary configuration alone and print its figures "
                         "(for profiler captures)")
    ap.add_argument("--c4-groups", type=int, default=8192, help="signal groups of C4 (8 signals each)")
    ap.add_argument("--c2-images", type=int, default=4096, help="images of C2 (a smaller batch for profiler captures)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    global W, H, J, WORKLOAD, SERVE_SECONDS
    SERVE_SECONDS = args.serve_seconds
    if args.image != 16384:
        W = H = args.image
        J = int(np.ceil(np.log2(W)))
        WORKLOAD = f"cdf97 2D forward+inverse, {W}x{H} float32, j_max={J}"

    ws, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return

    import torch
    import libdwt_gb300 as D

    torch.cuda.set_device(local)
    D.lib()
    if args.only:
        stream = torch.cuda.current_stream()
        checks = {}
        if args.only == "c4":
            res = run_signals_extra(D, torch, checks, groups=args.c4_groups)
        elif args.only == "c2":
            res = run_batch_extra(D, torch, stream, stream.cuda_stream, checks, n_images=args.c2_images)
        elif args.only == "dropin":
            res = run_dropin_extra(D, torch, torch.from_numpy(synth_image()).cuda(), args.dropin_reps)
        elif args.only == "dropin-dense":
            res = run_dropin_extra(D, torch, torch.from_numpy(synth_image()).cuda(), args.dropin_reps,
                                   parts=("dense",))
        elif args.only == "sparse":
            res = run_dropin_extra(D, torch, None, args.dropin_reps, parts=("sparse",))
        else:
            res = run_serve_extra(D, torch, SERVE_SECONDS)
        print(json.dumps({"only": args.only, **res}), flush=True)
        return
    img = synth_image()
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream

    src = torch.from_numpy(img).cuda()
    coef = torch.empty_like(src)
    rec = torch.empty_like(src)

    def step():
        D.transform2_dev(src, coef, "cdf97", False, J, 0, sptr)
        D.transform2_dev(coef, rec, "cdf97", True, J, 0, sptr)

    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier(ws)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    tw0 = time.time()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    tw1 = time.time()
    barrier(ws)
    ms = e0.elapsed_time(e1)
    ms = allmax(ws, ms)
    if D.lib().dwt_gpu_sync_check() != 0:
        raise SystemExit("device error during the timed region")
    px_step = 2 * W * H
    value = replica_value(ws, args.steps, px_step, ms)
    # algorithmic bytes of one step: 8 B per pixel of every level, both
    # directions
    step_bytes = 2 * sum(8 * (-(-W // (1 << k))) * (-(-H // (1 << k))) for k in range(J))

    # parity spot check of the benchmarked output (outside the timed region):
    # the reconstruction is within the reference's round-trip tolerance
    err_rt = float((rec - src).abs().max().item())

    # level 0 alone, both directions (16384^2 <-> four bands), each timed
    # with CUDA events over `reps` back-to-back launches.  The dominant
    # kernel is the level-kernel instance with the larger share of the step:
    # the instance of the slower direction (it runs every level of its
    # direction but the coarse ones), timed here as whole transforms
    bands = torch.empty_like(src)
    ll = torch.empty((H // 2, W // 2), dtype=torch.float32, device="cuda")
    rec0 = torch.empty_like(src)
    hw, hh = W // 2, H // 2
    outs = [ll.data_ptr(), bands.data_ptr() + hw * 4, bands.data_ptr() + hh * W * 4,
            bands.data_ptr() + (hh * W + hw) * 4]
    pitches = [hw * 4, W * 4, W * 4, W * 4]
    reps = max(1, args.level_reps)

    def level0(inverse):
        if inverse:
            D.level_dev("cdf97", True, W, H, outs, pitches, [rec0.data_ptr()], [W * 4], sptr)
        else:
            D.level_dev("cdf97", False, W, H, [src.data_ptr()], [W * 4], outs, pitches, sptr)

    level_ms = {}
    tk0 = time.time()
    for inverse in (False, True):
        for _ in range(3):
            level0(inverse)
        torch.cuda.synchronize()
        k0 = torch.cuda.Event(enable_timing=True)
        k1 = torch.cuda.Event(enable_timing=True)
        k0.record(stream)
        for _ in range(reps):
            level0(inverse)
        k1.record(stream)
        torch.cuda.synchronize()
        level_ms[inverse] = k0.elapsed_time(k1) / reps
    dir_ms = {}
    for inverse in (False, True):
        a, b_ = (src, coef) if not inverse else (coef, rec)
        for _ in range(2):
            D.transform2_dev(a, b_, "cdf97", inverse, J, 0, sptr)
        torch.cuda.synchronize()
        k0 = torch.cuda.Event(enable_timing=True)
        k1 = torch.cuda.Event(enable_timing=True)
        k0.record(stream)
        for _ in range(5):
            D.transform2_dev(a, b_, "cdf97", inverse, J, 0, sptr)
        k1.record(stream)
        torch.cuda.synchronize()
        dir_ms[inverse] = k0.elapsed_time(k1) / 5
    tk1 = time.time()
    level0_rt_err = float((rec0 - src).abs().max().item())  # one level forward, then inverse
    dom_inv = dir_ms[True] >= dir_ms[False]
    kms = level_ms[dom_inv]
    alg_bytes = 8 * W * H
    achieved = alg_bytes / (kms / 1e3) / 1e9
    peak, peak_kind = hbm_peak()
    traffic = None
    tfile = os.path.join(ROOT, "profiles", "level0_traffic.json")
    if os.path.exists(tfile):
        with open(tfile) as f:
            tj = json.load(f)
        traffic = tj.get("inverse" if dom_inv else "forward", {}).get("dram_bytes_per_launch")

    # e2e through the drop-in C ABI on a pinned host image
    if args.skip_e2e:
        e2e_value, e2e_steps, err_e2e = None, 0, None
    else:
        e2e_value, e2e_steps, err_e2e = run_e2e(D, torch, img, args, ws)

    checks = {}
    extras = {}
    if not args.no_extras:
        extras = run_extras(D, torch, stream, sptr, checks)
    sampler.stop()
    clocks = sampler.summary(tw0, tw1)

    cpu, errors = None, None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        # the CPU leg: the timed restatement, then the FP64 error checks
        from oracle import oracle as O
        threads = O.max_threads()
        mpx, desc = cpu_baseline(img, threads)
        cpu = {"value": round(mpx, 3), "unit": "Mpx/s", "cores": threads, "kind": "port", "sample": desc,
               "pin": ("the reference itself at accel 9 runs this workload at 1.03x the port's rate (x86, same "
                       "threads, bit-identical outputs; profiles/cpu_reference_vs_port_x86.md)")}
        D.transform2_dev(src, coef, "cdf97", False, J, 0, sptr)
        D.transform2_dev(coef, rec, "cdf97", True, J, 0, sptr)
        torch.cuda.synchronize()
        errors = cpu_checks(threads, img, coef.cpu().numpy(), rec.cpu().numpy(), checks)
        cpu["configs"] = cpu_configs(threads)

    if rank == 0:
        line = {
            "metric": "2D DWT throughput (CDF 9/7 forward+inverse, full depth)",
            "value": round(value, 1), "unit": "Mpx/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded 64-blob field + N(0,4) noise, integers 0..255)",
            "config": {"workload": WORKLOAD, "image": [W, H], "j_max": J,
                       "l2": "inputs (1 GiB) larger than L2, no flush",
                       "parallelism": "replicas" if ws > 1 else "single GPU"},
            "e2e": None if e2e_value is None else {"value": round(e2e_value, 1), "unit": "Mpx/s", "steps": e2e_steps,
                    "h2d_bytes_per_step": 2 * W * H * 4, "d2h_bytes_per_step": 2 * W * H * 4,
                    "api": "dwt_cdf97_2f_s + dwt_cdf97_2i_s on pinned host memory",
                    "roundtrip_max_abs_err": err_e2e},
            "roofline": {"bound": "hbm",
                         "kernel": ("level_kernel<4,true> (CDF 9/7 inverse, level 0)" if dom_inv
                                    else "level_kernel<4,false> (CDF 9/7 forward, level 0)"),
                         "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                         "traffic": traffic, "algorithmic_bytes_per_launch": alg_bytes,
                         "launch_ms": round(kms, 4),
                         "other_level0": {
                             "kernel": ("level_kernel<4,false> (CDF 9/7 forward, level 0)" if dom_inv
                                        else "level_kernel<4,true> (CDF 9/7 inverse, level 0)"),
                             "launch_ms": round(level_ms[not dom_inv], 4),
                             "frac": round(alg_bytes / (level_ms[not dom_inv] / 1e3) / 1e9 / peak, 4)},
                         "direction_ms": {"forward": round(dir_ms[False], 4), "inverse": round(dir_ms[True], 4)},
                         "level0_roundtrip_max_abs_err": level0_rt_err,
                         "step_bytes": step_bytes,
                         "step_frac": round(step_bytes / (ms / args.steps / 1e3) / 1e9 / peak, 4)},
            "cpu_baseline": cpu,
            "clocks": clocks,
            "gpu_launches": args.steps * 2 * D.lib().dwt_gpu_dense_launches(W, H, J),
            "roundtrip_max_abs_err": err_rt,
            "errors_vs_fp64": errors,
            "extras": extras,
        }
        print(json.dumps(line), flush=True)


def run_dropin_extra(D, torch, src, nd=10, parts=("dense", "sparse", "dense12000")):
    """The drop-in calls themselves on device pointers, in place as the
    reference's callers use them (synchronous calls): CDF 9/7 forward +
    inverse of the 16384^2 image, and of a 12000^2 image in a 16384^2 outer
    frame with zero padding (the OpenCV wrapper's power-of-two padding;
    Mpx/s of inner pixels)."""
    out = {}
    if "dense" in parts:
        out.update(_dropin_dense(D, torch, src, nd))
    if "sparse" in parts:
        out.update(_dropin_sparse(D, torch, nd))
    if "dense12000" in parts:
        out.update(_dropin_dense12000(D, torch, nd))
    return out


def _dropin_dense(D, torch, src, nd):
    out = {}
    # the drop-in itself on a device pointer (in place, as the reference's
    # callers use it; synchronous calls), forward + inverse of 16384^2
    dimg = src.clone()
    dp = dimg.data_ptr()
    for _ in range(2):
        jd = D.dwt_cdf97_2f_s(dp, W * 4, 4, W, H, W, H, J)
        D.dwt_cdf97_2i_s(dp, W * 4, 4, W, H, W, H, jd)
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(nd):
        jd = D.dwt_cdf97_2f_s(dp, W * 4, 4, W, H, W, H, J)
        D.dwt_cdf97_2i_s(dp, W * 4, 4, W, H, W, H, jd)
    dt = time.perf_counter() - t
    out["c1_dropin_device_mpx_s"] = round(nd * 2 * W * H / dt / 1e6, 1)
    out["c1_dropin_device_ms_per_pair"] = round(dt / nd * 1e3, 3)
    out["c1_dropin_device_roundtrip_max_abs_err"] = float((dimg - src).abs().max().item())
    del dimg
    return out


def _dropin_sparse(D, torch, nd):
    from libdwt_gb300 import synth
    out = {}
    # a sparse frame: a 12000^2 image in a 16384^2 outer frame with zero
    # padding (the OpenCV wrapper's power-of-two padding), drop-in forward +
    # inverse in place on the device; Mpx/s of inner pixels
    sp = torch.zeros((H, W), dtype=torch.float32, device="cuda")
    sp[:12000, :12000] = torch.from_numpy(synth.image(12000, 12000, seed=9)).cuda()
    spp = sp.data_ptr()
    for _ in range(2):
        js = D.dwt_cdf97_2f_s(spp, W * 4, 4, W, H, 12000, 12000, -1, 0, 1)
        D.dwt_cdf97_2i_s(spp, W * 4, 4, W, H, 12000, 12000, js, 0, 1)
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(nd):
        js = D.dwt_cdf97_2f_s(spp, W * 4, 4, W, H, 12000, 12000, -1, 0, 1)
        D.dwt_cdf97_2i_s(spp, W * 4, 4, W, H, 12000, 12000, js, 0, 1)
    dt = time.perf_counter() - t
    out["c1_sparse_12000_in_16384_dropin_device_mpx_s"] = round(nd * 2 * 12000 * 12000 / dt / 1e6, 1)
    del sp
    return out


def _dropin_dense12000(D, torch, nd):
    from libdwt_gb300 import synth
    out = {}
    # the same 12000^2 image as a dense frame (outer = inner), same calls:
    # the rate the sparse frame is compared with, per inner pixel
    de = torch.from_numpy(synth.image(12000, 12000, seed=9)).cuda()
    dep = de.data_ptr()
    for _ in range(2):
        js = D.dwt_cdf97_2f_s(dep, 12000 * 4, 4, 12000, 12000, 12000, 12000, -1)
        D.dwt_cdf97_2i_s(dep, 12000 * 4, 4, 12000, 12000, 12000, 12000, js)
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(nd):
        js = D.dwt_cdf97_2f_s(dep, 12000 * 4, 4, 12000, 12000, 12000, 12000, -1)
        D.dwt_cdf97_2i_s(dep, 12000 * 4, 4, 12000, 12000, 12000, 12000, js)
    dt = time.perf_counter() - t
    out["c1_dense_12000_dropin_device_mpx_s"] = round(nd * 2 * 12000 * 12000 / dt / 1e6, 1)
    del de
    return out


def run_e2e(D, torch, img, args, ws):
    """Forward + inverse through the drop-in C ABI on a pinned host image; the
    calls copy the image in and the result out every time."""
    host = torch.from_numpy(img.copy()).pin_memory()
    hp = host.data_ptr()
    e2e_steps = max(3, min(args.steps, 10))
    for _ in range(2):
        j = D.dwt_cdf97_2f_s(hp, W * 4, 4, W, H, W, H, J)
        D.dwt_cdf97_2i_s(hp, W * 4, 4, W, H, W, H, j)
    barrier(ws)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        j = D.dwt_cdf97_2f_s(hp, W * 4, 4, W, H, W, H, J)
        D.dwt_cdf97_2i_s(hp, W * 4, 4, W, H, W, H, j)
    e2e_s = allmax(ws, time.perf_counter() - t0)
    e2e_value = ws * e2e_steps * 2 * W * H / e2e_s / 1e6
    err_e2e = float(np.abs(host.numpy() - img).max())
    return e2e_value, e2e_steps, err_e2e


def run_extras(D, torch, stream, sptr, checks: dict):
    """Secondary figures of the other configurations (outside the headline);
    GPU outputs for the CPU leg's error checks are left in `checks`."""
    out = {}
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)

    def timed(fn, reps):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(reps):
            fn()
        ev1.record(stream)
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1) / reps

    from libdwt_gb300 import synth
    img = synth_image()
    src = torch.from_numpy(img).cuda()
    dst = torch.empty_like(src)
    for wav in ("cdf97", "cdf53"):
        for inv in (False, True):
            ms = timed(lambda: D.transform2_dev(src, dst, wav, inv, J, 0, sptr), 10)
            out[f"{wav}_{'inv' if inv else 'fwd'}_16384_mpx_s"] = round(W * H / ms / 1e3, 1)
            out[f"{wav}_{'inv' if inv else 'fwd'}_16384_frac_alg"] = round(
                2863311520 / (ms / 1e3) / 1e9 / hbm_peak()[0], 4)
    # odd size: 16383 x 16385 (rows padded to a 16-byte pitch)
    ow, oh = 16383, 16385
    osrc = torch.zeros((oh, 16384), dtype=torch.float32, device="cuda")
    osrc[:, :ow] = torch.from_numpy(synth.image(ow, oh, seed=1)).cuda()
    odst = torch.empty((oh, ow), dtype=torch.float32, device="cuda")
    for wav in ("cdf97", "cdf53"):
        ms = timed(lambda: D.transform2_dev(osrc[:, :ow], odst, wav, False, J, 0, sptr), 10)
        out[f"{wav}_fwd_16383x16385_mpx_s"] = round(ow * oh / ms / 1e3, 1)
    del osrc, odst
    out.update(run_dropin_extra(D, torch, src))
    # plain drop-in latency, 1024^2 j=5 on a host image (forward + inverse)
    small = synth.image(1024, 1024, seed=2)
    t = time.perf_counter()
    n = 20
    for _ in range(n):
        j = D.dwt_cdf97_2f_s(small.ctypes.data, 4096, 4, 1024, 1024, 1024, 1024, 5)
        D.dwt_cdf97_2i_s(small.ctypes.data, 4096, 4, 1024, 1024, 1024, 1024, j)
    out["c0_1024_fwd_inv_host_ms"] = round((time.perf_counter() - t) / n * 1e3, 3)
    # the drop-in on a pageable (malloc'ed) 16384^2 host image, as the
    # reference's callers allocate it: forward + inverse, 3 steps after one
    page = synth.image(16384, 16384, seed=3)
    pp = page.ctypes.data
    j = D.dwt_cdf97_2f_s(pp, 16384 * 4, 4, 16384, 16384, 16384, 16384, -1)
    D.dwt_cdf97_2i_s(pp, 16384 * 4, 4, 16384, 16384, 16384, 16384, j)
    t = time.perf_counter()
    for _ in range(3):
        j = D.dwt_cdf97_2f_s(pp, 16384 * 4, 4, 16384, 16384, 16384, 16384, -1)
        D.dwt_cdf97_2i_s(pp, 16384 * 4, 4, 16384, 16384, 16384, 16384, j)
    out["e2e_pageable_16384_mpx_s"] = round(3 * 2 * 16384 * 16384 / (time.perf_counter() - t) / 1e6, 1)
    del page
    dsmall = torch.from_numpy(small).cuda()

    def c0dev():
        j = D.dwt_cdf97_2f_s(dsmall.data_ptr(), 4096, 4, 1024, 1024, 1024, 1024, 5)
        D.dwt_cdf97_2i_s(dsmall.data_ptr(), 4096, 4, 1024, 1024, 1024, 1024, j)
    c0dev()
    t = time.perf_counter()
    for _ in range(n):
        c0dev()
    out["c0_1024_fwd_inv_device_ms"] = round((time.perf_counter() - t) / n * 1e3, 3)
    small0 = synth.image(1024, 1024, seed=2)
    c0 = torch.from_numpy(small0).cuda()
    c0_out = torch.empty_like(c0)
    D.transform2_dev(c0, c0_out, "cdf97", False, 5, 0, sptr)
    torch.cuda.synchronize()
    checks["c0"] = (small0, c0_out.cpu().numpy())
    out.update(run_signals_extra(D, torch, checks))
    out.update(run_batch_extra(D, torch, stream, sptr, checks))
    out.update(run_serve_extra(D, torch, SERVE_SECONDS))
    return out


SERVE_SECONDS = 10.0


def serve_trace(seconds: float, rate: float = 20000.0, seed: int = 11):
    """Poisson arrivals (mean `rate` per second) of forward or inverse 2D
    transforms: area log-uniform in 32^2..8192^2, aspect ratio uniform in
    [0.5, 2], CDF 9/7 or 5/3 and direction 50/50, j_max uniform in 1..6."""
    rng = np.random.default_rng(seed)
    n = int(rate * seconds * 1.1) + 16
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    t = t[t < seconds]
    n = len(t)
    area = np.exp(rng.uniform(np.log(32 * 32), np.log(8192 * 8192), n))
    a = rng.uniform(0.5, 2.0, n)
    w = np.maximum(1, np.rint(np.sqrt(area * a))).astype(int)
    h = np.maximum(1, np.rint(np.sqrt(area / a))).astype(int)
    wav = rng.integers(0, 2, n)
    inv = rng.integers(0, 2, n)
    j = rng.integers(1, 7, n)
    return t, w, h, wav, inv, j


def run_serve_extra(D, torch, seconds: float):
    """Serving loop: a 20k req/s Poisson stream replayed in real time against
    the continuous-batching server (64 GiB admission budget, pooled buffers,
    8 streams);
    every request reads its w x h input from a resident synthetic image and
    writes its result to a pooled buffer."""
    from libdwt_gb300 import synth
    t, w, h, wav, inv, j = serve_trace(seconds)
    side = int(max(w.max(), h.max()))
    pitch = (side + 3) // 4 * 4
    src = torch.empty((side, pitch), dtype=torch.float32, device="cuda")
    src[:, :side] = synth.image_torch(side, side, seed=5)
    torch.cuda.synchronize()
    reqs = [D.Server.request(src, None, "cdf97" if wav[k] == 0 else "cdf53", bool(inv[k]), int(j[k]), tag=k,
                             w=int(w[k]), h=int(h[k])) for k in range(len(t))]
    srv = D.Server(budget_bytes=64 << 30, n_streams=8)
    # set-up outside the measured replay: the arena's device memory and one
    # request of every path, so no allocation or kernel loading happens
    # while requests are served
    t0 = time.perf_counter()
    srv.reserve(16 << 30)
    reserve_s = time.perf_counter() - t0
    st0 = srv.stats()
    t0 = time.perf_counter()
    lat = srv.replay(t, reqs, timeout_s=600)
    wall = time.perf_counter() - t0
    st = srv.stats()
    px = float((w.astype(np.int64) * h).sum())
    res = {"c3_seconds": seconds, "c3_requests": int(len(t)), "c3_offered_mpx_s": round(px / seconds / 1e6, 1),
           "c3_sustained_mpx_s": round(px / wall / 1e6, 1), "c3_p50_ms": round(float(np.percentile(lat, 50)) * 1e3, 3),
           "c3_p99_ms": round(float(np.percentile(lat, 99)) * 1e3, 3),
           "c3_max_ms": round(float(lat.max()) * 1e3, 3), "c3_launches": st["launches"],
           "c3_peak_bytes": st["peak_bytes"], "c3_budget_bytes": st["budget_bytes"],
           "c3_reserve_s": round(reserve_s, 3), "c3_arena_bytes": st["arena_bytes"],
           "c3_device_allocs_in_replay": st["device_allocs"] - st0["device_allocs"],
           "c3_max_dispatch_ms": round(st["max_dispatch_ns"] / 1e6, 3)}
    # capacity: the first 2 s of the same trace offered 5x faster (100k req/s)
    k2 = int(np.searchsorted(t, 2.0))
    t0 = time.perf_counter()
    lat2 = srv.replay(t[:k2] / 5.0, reqs[:k2], timeout_s=600)
    wall2 = time.perf_counter() - t0
    px2 = float((w[:k2].astype(np.int64) * h[:k2]).sum())
    srv.close()
    res.update({"c3_x5_offered_mpx_s": round(px2 / (t[k2 - 1] / 5.0) / 1e6, 1),
                "c3_x5_sustained_mpx_s": round(px2 / wall2 / 1e6, 1),
                "c3_x5_p50_ms": round(float(np.percentile(lat2, 50)) * 1e3, 3),
                "c3_x5_p99_ms": round(float(np.percentile(lat2, 99)) * 1e3, 3)})
    # the plain per-request drop-in on the first 2000 requests of the mix
    # (in place on a device copy of each input, one synchronous call each)
    n3 = min(2000, len(t))
    work = []
    for k in range(n3):
        work.append(src[: int(h[k]), : int(w[k])].clone())
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(n3):
        ww, hh = int(w[k]), int(h[k])
        x = work[k]
        if inv[k]:
            (D.dwt_cdf97_2i_s if wav[k] == 0 else D.dwt_cdf53_2i_s)(x.data_ptr(), ww * 4, 4, ww, hh, ww, hh, int(j[k]))
        else:
            (D.dwt_cdf97_2f_s if wav[k] == 0 else D.dwt_cdf53_2f_s)(x.data_ptr(), ww * 4, 4, ww, hh, ww, hh, int(j[k]))
    torch.cuda.synchronize()
    px3 = float((w[:n3].astype(np.int64) * h[:n3]).sum())
    res["c3_plain_dropin_mpx_s"] = round(px3 / (time.perf_counter() - t0) / 1e6, 1)
    res["c3_capacity_vs_plain"] = round(res["c3_x5_sustained_mpx_s"] / res["c3_plain_dropin_mpx_s"], 1)
    return res


def run_signals_extra(D, torch, checks: dict, groups=8192, n=4097, lanes=8):
    """Strided 1D lifting: 65536 AR(1) signals of 4097 samples, 8 interleaved
    per group (element stride 32 B), CDF 9/7 forward then inverse, one batched
    in-place launch each (dwt_gpu_1_batch_s on device memory)."""
    from libdwt_gb300 import synth
    x = synth.ar1_bank(groups, n, lanes, seed=4)
    dev = torch.from_numpy(x).cuda()
    gs, st, count = n * lanes * 4, lanes * 4, groups * lanes

    def fwd():
        D.batch_1d("cdf97", False, dev, n, st, count, lanes, gs, 4)

    def inv():
        D.batch_1d("cdf97", True, dev, n, st, count, lanes, gs, 4)
    fwd()
    inv()
    torch.cuda.synchronize()
    reps = 5
    t0 = time.perf_counter()
    for _ in range(reps):
        fwd()
    tf = (time.perf_counter() - t0) / reps
    t0 = time.perf_counter()
    for _ in range(reps):
        inv()
    ti = (time.perf_counter() - t0) / reps
    samples = groups * lanes * n
    percall = c4_per_call(D, torch, x, n, lanes)
    # one forward pass on a slice, checked in the CPU leg
    part = x[:64].copy()
    dpart = torch.from_numpy(part).cuda()
    D.batch_1d("cdf97", False, dpart, n, st, 64 * lanes, lanes, gs, 4)
    checks["c4"] = (part, dpart.cpu().numpy(), n, st, 64 * lanes, lanes, gs)
    peak = hbm_peak()[0]
    return {"c4_signals": count, "c4_n": n, "c4_fwd_ms": round(tf * 1e3, 3), "c4_inv_ms": round(ti * 1e3, 3),
            "c4_fwd_gsamples_s": round(samples / tf / 1e9, 2), "c4_inv_gsamples_s": round(samples / ti / 1e9, 2),
            "c4_fwd_frac_alg": round(8 * samples / tf / 1e9 / peak, 4),
            "c4_inv_frac_alg": round(8 * samples / ti / 1e9 / peak, 4), **percall}


def native_calls_1d():
    """The OpenMP driver of the per-signal calls (libdwt_gb300/harness/calls_1d.c),
    built against the library on first use; None when it cannot be built."""
    import ctypes as C
    import shutil
    import subprocess
    from libdwt_gb300.buildext import LIB
    src = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libdwt_gb300", "harness", "calls_1d.c")
    out = os.path.join(os.path.dirname(LIB), "libcalls_1d.so")
    cc = shutil.which("gcc")
    if not cc or not os.path.exists(src):
        return None
    if not os.path.exists(out) or os.path.getmtime(out) < max(os.path.getmtime(src), os.path.getmtime(LIB)):
        r = subprocess.run([cc, "-O2", "-fopenmp", "-shared", "-fPIC", src, "-o", out, "-L", os.path.dirname(LIB),
                            "-l:" + os.path.basename(LIB), "-Wl,-rpath," + os.path.dirname(LIB)],
                           capture_output=True, text=True)
        if r.returncode != 0:
            return None
    lib = C.CDLL(out)
    lib.calls_1d.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_longlong, C.c_longlong, C.c_int]
    lib.calls_1d.restype = C.c_double
    return lib


def c4_per_call(D, torch, bank, n, lanes, n_groups=512, threads=16):
    """The reference's own calling pattern for the signal bank, against this
    library: `threads` host threads, each calling the drop-in
    dwt_cdf97_f_ex_stride_s once per signal of its share (in place, L at the
    signal's start, H ceil(N/2) samples later, element stride 32 B), on the
    first `n_groups` groups of the bank -- in the reference's host memory
    (malloc'ed) and on a device copy.  Reports Gsamples/s and microseconds
    per call, beside the batched launch's figures."""
    import ctypes as C
    import threading
    L = D.lib()
    f = L.dwt_cdf97_f_ex_stride_s
    part = np.ascontiguousarray(bank[:n_groups]).copy()
    dev = torch.from_numpy(part).cuda()
    count = n_groups * lanes
    st, gs = lanes * 4, n * lanes * 4
    off_h = ((n + 1) // 2) * st
    out = {}
    for where, base in (("host", part.ctypes.data), ("device", dev.data_ptr())):
        def work(k0, k1):
            for s in range(k0, k1):
                a = base + (s // lanes) * gs + (s % lanes) * 4
                f(a, a, a + off_h, None, n, st)
        f(base, base, base + off_h, None, n, st)  # first call outside the timing
        torch.cuda.synchronize()
        ths = [threading.Thread(target=work, args=(count * t // threads, count * (t + 1) // threads))
               for t in range(threads)]
        t0 = time.perf_counter()
        for th in ths:
            th.start()
        for th in ths:
            th.join()
        dt = time.perf_counter() - t0
        out[f"c4_dropin_per_call_{where}_gsamples_s"] = round(count * n / dt / 1e9, 4)
        out[f"c4_dropin_per_call_{where}_us"] = round(dt / count * threads * 1e6, 1)
    out["c4_dropin_per_call_sample"] = (f"{count} signals of {n} (the first {n_groups} groups), {threads} host "
                                        f"threads, one dwt_cdf97_f_ex_stride_s call per signal")
    # the same calls from native code: an OpenMP loop, as the reference's callers run it
    nat = native_calls_1d()
    if nat is not None:
        for where, base in (("host", part.ctypes.data), ("device", dev.data_ptr())):
            nat.calls_1d(0, base, n, st, lanes, gs, lanes, threads)  # warm-up
            torch.cuda.synchronize()
            dt = nat.calls_1d(0, base, n, st, lanes, gs, count, threads)
            out[f"c4_dropin_per_call_openmp_{where}_gsamples_s"] = round(count * n / dt / 1e9, 4)
            out[f"c4_dropin_per_call_openmp_{where}_us"] = round(dt / count * threads * 1e6, 1)
    return out


def run_batch_extra(D, torch, stream, sptr, checks: dict, n_images=4096, j=4):
    """Batched uneven images: 4096 images, sides log-uniform in 33..2048, CDF
    9/7 or 5/3 per image, j_max = 4, forward.  The autotuned persistent graph
    against the plain per-image drop-in (dwt_cdf97_2f_s / dwt_cdf53_2f_s on
    device pointers, one call per image) on the same device data."""
    from libdwt_gb300 import synth
    sizes = synth.batch_sizes(n_images, seed=7)
    srcs, dsts, imgs = [], [], []
    total_px = 0
    for k, (w, h, wav) in enumerate(sizes):
        pw = (w + 3) // 4 * 4
        buf = torch.empty((h, pw), dtype=torch.float32, device="cuda")
        buf[:, :w] = synth.image_torch(w, h, seed=1000 + k)
        src = buf[:, :w]
        dst = torch.empty((h, w), dtype=torch.float32, device="cuda")
        srcs.append(src)
        dsts.append(dst)
        imgs.append(dict(src=src, dst=dst, wavelet="cdf97" if wav == 0 else "cdf53", inverse=False,
                         j_levels=j))
        total_px += w * h
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b = D.Batch(imgs, None)
    plan_s = time.perf_counter() - t0
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    b.run(sptr)
    torch.cuda.synchronize()
    reps = 10
    ev0.record(stream)
    for _ in range(reps):
        b.run(sptr)
    ev1.record(stream)
    torch.cuda.synchronize()
    batch_ms = ev0.elapsed_time(ev1) / reps
    # plain drop-in: in place on a device copy of every input, one call each
    work = [s.clone() for s in srcs]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k, (w, h, wav) in enumerate(sizes):
        f = D.dwt_cdf97_2f_s if wav == 0 else D.dwt_cdf53_2f_s
        f(work[k].data_ptr(), work[k].stride(0) * 4, 4, w, h, w, h, j)
    torch.cuda.synchronize()
    plain_s = time.perf_counter() - t0
    maxdiff = 0.0
    for k in range(len(sizes)):
        maxdiff = max(maxdiff, float((work[k] - dsts[k]).abs().max().item()))
    # the inverse of every image in one batch of its own: the round trip of
    # all 4096 images on the device
    backs, inv_imgs = [], []
    for k, (w, h, wav) in enumerate(sizes):
        pw = (w + 3) // 4 * 4
        cbuf = torch.empty((h, pw), dtype=torch.float32, device="cuda")
        cbuf[:, :w] = dsts[k]
        back = torch.empty((h, w), dtype=torch.float32, device="cuda")
        backs.append(back)
        inv_imgs.append(dict(src=cbuf[:, :w], dst=back, wavelet="cdf97" if wav == 0 else "cdf53", inverse=True,
                             j_levels=j))
    bi = D.Batch(inv_imgs, b.params)
    bi.run(sptr)
    torch.cuda.synchronize()
    rt_err = max(float((backs[k] - srcs[k]).abs().max().item()) for k in range(len(sizes)))
    bi.close()
    # 32 images of the batch for the CPU leg's FP64 check (forward and round trip)
    sample = []
    for k in range(0, len(sizes), max(1, len(sizes) // 32))[:32]:
        w, h, wav = sizes[k]
        sample.append((srcs[k].cpu().numpy().copy(), dsts[k].cpu().numpy(), "cdf97" if wav == 0 else "cdf53", j,
                       backs[k].cpu().numpy()))
    checks["c2"] = sample
    del backs, inv_imgs
    res = {"c2_images": n_images, "c2_pixels": total_px, "c2_batch_mpx_s": round(total_px / batch_ms / 1e3, 1),
           "c2_batch_ms": round(batch_ms, 3), "c2_plain_dropin_mpx_s": round(total_px / plain_s / 1e6, 1),
           "c2_speedup_vs_plain": round((total_px / batch_ms / 1e3) / (total_px / plain_s / 1e6), 1),
           "c2_max_abs_diff_vs_plain": maxdiff, "c2_autotuned_params": list(b.params),
           "c2_roundtrip_max_abs_err_all_images": rt_err,
           "c2_items": b.items, "c2_plan_s": round(plan_s, 2)}
    b.close()
    return res


if __name__ == "__main__":
    main()
