#!/usr/bin/env python3
"""Benchmark of the xc_fast hot path on one GB300 (replicas on N GPUs).

Workload (the precision configuration): 64 stations x 3 components x 30 days
at delta 0.1 s, win_len 3600 s -> 720 windows of 36 000 samples, output
spectra of nspec = 18 523 bins (output_nfft 37 044), all 2016 station pairs
x 9 component pairs = 18 144 pairs, 5 % of windows zeroed as gaps, linear
stack over all windows, max_lag 100 s -> 2001 lags per NCF.

One step = correlate + stack all 18 144 pairs over the 720 windows, then the
C2R + lag cut: 13 063 680 pair-windows. Inputs (20.5 GB of spectra) are
resident in HBM and larger than L2 (no L2 flush needed).

Metric: pair-windows/s. `value` is the device-resident throughput of the
selected method (tensor-core BF16 hi/lo when built, else plain FP32);
`e2e` runs the same step through the host-buffer C-ABI call
(fxc_xc_run_host) with the H2D copy of the spectra and the D2H copy of the
NCFs inside the timed region.

`--impl reference` times the FP64 CPU oracle (the reference algorithm
restated; the reference itself has no CPU path and its CUDA sources do not
exist on the GPU host) on a bounded sample of the same workload, using all
host cores.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

NSTA, NCOMP, NDAYS, NSTEP = 64, 3, 30, 24
DT, CC_LEN = 0.1, 100.0
NSPEC = 18523  # output_nfft 37044 / 2 + 1 for win_len 3600 s, lag 100 s at 10 Hz
GAP_FRAC = 0.05


LAYOUT_NAMES = {0: "auto", 1: "whole_bin", 2: "tiled"}

def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--method", default="auto", choices=["auto", "plain", "tensor"])
    ap.add_argument("--days", type=int, default=NDAYS)
    ap.add_argument("--nspec", type=int, default=NSPEC, help="smaller values only for profiling runs")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-stages", action="store_true", help="skip the sac2spec / stacking stage timings")
    ap.add_argument("--stack-pairs", type=int, default=2304, help="pairs of the stacking stages; smaller values only for profiling runs")
    ap.add_argument("--batch-block", type=int, default=0, help="unused; kept for older command lines")
    ap.add_argument("--batch-days", type=int, default=10, help="days of the batching stage")
    ap.add_argument("--serve-seconds", type=float, default=8.0, help="serving stream length; 0 skips it")
    ap.add_argument("--profile-case", choices=["sac2spec", "stacking"], default=None,
                    help="run one small case of a stage (for ncu captures) and exit")
    ap.add_argument("--serve-rate", type=float, default=20.0)
    ap.add_argument("--serve-slots", type=int, default=4)
    ap.add_argument("--serve-wait-limit", type=float, default=240.0)
    return ap.parse_args()


def dist_env():
    from fastxc_gb300.replicas import dist_env as env

    rank, world, local = env()
    return rank, world, local


class ClockSampler:
    """nvidia-smi sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_model() -> str:
    """CPU model name of the host (lscpu, else /proc/cpuinfo, else the
    machine type)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for ln in Path("/proc/cpuinfo").read_text().splitlines():
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform

    return platform.machine()


def cpu_baseline(seconds_target=15.0, threads=1):
    """FP64 oracle on a bounded sample: 16 stations (48 channels), whole days
    of 24 windows, all 9 x 120 component pairs; returns pair-windows/s."""
    from concurrent.futures import ThreadPoolExecutor

    from fastxc_gb300.synthetic import cross_station_pairs
    from oracle import xc_oracle as xo

    rng = np.random.default_rng(1)
    nsta, nwin = 16, NSTEP
    nchan = nsta * NCOMP
    spec = (rng.standard_normal((nwin, nchan, NSPEC)) + 1j * rng.standard_normal((nwin, nchan, NSPEC))).astype(np.complex64)
    src, rec = cross_station_pairs(nsta)
    shape = xo.finalize_shape(NSPEC, nwin, DT, CC_LEN)
    chunks = np.array_split(np.arange(src.size), max(1, threads))

    def work(idx):
        xo.xc_run(spec, src[idx], rec[idx], 1.0 / nwin, shape)

    done_pw = 0
    t0 = time.perf_counter()
    reps = 0
    while True:
        if threads == 1:
            work(np.arange(src.size))
        else:
            with ThreadPoolExecutor(threads) as ex:
                list(ex.map(work, chunks))
        reps += 1
        done_pw += src.size * nwin
        if time.perf_counter() - t0 > seconds_target:
            break
    el = time.perf_counter() - t0
    return done_pw / el, f"{reps} x (16 stations x 3 comps, 1 day = 24 windows, {src.size} pairs, nspec {NSPEC}), FP64 numpy"


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    per_step = []
    sample = ""
    for i in range(args.warmup + args.steps):
        v, sample = cpu_baseline(seconds_target=4.0, threads=cores)
        if i >= args.warmup:
            per_step.append(v)
    value = statistics.median(per_step)
    gpu_ref = reference_kernels_gpu()
    line = {
        "impl": "reference",
        "metric": "pair-windows/s",
        "value": value,
        "unit": "pair-windows/s",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": "xc linear stack, 64 sta x 3 comp x 30 days (sampled)", "nspec": NSPEC,
                   "pairs": 18144, "windows": NSTEP * NDAYS},
        "cpu_baseline": {"value": value, "unit": "pair-windows/s", "cores": cores, "kind": "port",
                         "sample": sample, "cpu_model": cpu_model()},
        "e2e": {"value": value, "unit": "pair-windows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if gpu_ref is not None:
        line["reference_kernels_gpu"] = gpu_ref
    print(json.dumps(line), flush=True)


def reference_kernels_gpu() -> dict | None:
    """The reference's own CUDA kernels (compiled from its sources with its
    release flags) and cuFFT, in its host order, timed on this GPU with CUDA
    events, inputs resident: one day of the precision configuration through
    xc (24 accumulate launches + sign flip + C2R + 1/(N dt)), one day of 64
    stations through sac2spec, PWS on 256 pairs and TF-PWS on 8 pairs of the
    stacking configuration. None when no GPU or the kernels are not built."""
    try:
        import torch

        if not torch.cuda.is_available():
            return None
        from oracle import ref_gpu
    except Exception:
        return None
    if not ref_gpu.available():
        return {"unavailable": "reference kernels not built (oracle/build_ref.py needs the reference tree)"}
    from fastxc_gb300.synthetic import cross_station_pairs, spectra_device, station_array
    from oracle import sac2spec_oracle as so
    from oracle import stack_oracle as sto

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream(dev)
    out = {"how": "reference kernel sources compiled by oracle/build_ref.py (-O3 --use_fast_math), cuFFT via torch "
                  "(each transform's result is copied once into the reference's pitched buffer), host order restated "
                  "in oracle/ref_gpu.py; CUDA events on the launching stream"}
    # xc: one day (24 windows) of 64 stations x 3 components, 18 144 pairs
    arr = station_array(NSTA, seed=0)
    src, rec = cross_station_pairs(NSTA)
    spec, _ = spectra_device(torch, NSTEP, arr, NSPEC, DT, seed=0, gap_frac=GAP_FRAC, device=dev)
    nfft = 2 * (NSPEC - 1)
    half = int(round(CC_LEN / DT))
    m = ref_gpu.RefModule.get("xc")
    d_src = torch.from_numpy(src.astype(np.int64)).to(dev)
    d_rec = torch.from_numpy(rec.astype(np.int64)).to(dev)
    stack = torch.zeros((src.size, NSPEC), dtype=torch.complex64, device=dev)
    sign = torch.zeros(NSPEC, dtype=torch.int32, device=dev)
    tim = torch.zeros((src.size, nfft), dtype=torch.float32, device=dev)
    ms = _timed(torch, stream, lambda: ref_gpu.xc_launch(m, spec, d_src, d_rec, stack, sign, tim, NSTEP, arr.nchan,
                                                         NSPEC, src.size, nfft, float(np.float32(DT)),
                                                         1.0 / NSTEP), reps=3, warm=1)
    out["xc_one_day"] = {"ms": ms, "pair_windows_per_s": src.size * NSTEP / (ms / 1e3), "pairs": int(src.size),
                         "windows": NSTEP, "nspec": NSPEC, "cc_size": 2 * half + 1}
    del spec, stack, tim
    torch.cuda.empty_cache()
    # sac2spec: one day of 64 stations x 3 components, RAM + whiten after
    op = so.make_plan(86400, 3600, 3600, 100, 0.1, so.read_filter_file(
        ROOT / "tests" / "golden" / "filter_d0.1_0.1-2.txt"), so.WHITEN_AFTER, so.NORM_RUNABS)
    rows = 192 * op.nstep
    g = torch.Generator(device=dev)
    g.manual_seed(7)
    x = torch.randn((rows, op.segment_pts), generator=g, device=dev, dtype=torch.float32)
    resp = torch.from_numpy(op.responses).to(dev)
    work = torch.empty_like(x)

    def s2s_once():
        work.copy_(x)
        ref_gpu.sac2spec_rows_device(work, op, resp, 3)

    ms = _timed(torch, stream, s2s_once, reps=2, warm=1)
    out["sac2spec_one_day"] = {"ms": ms, "channel_windows_per_s": rows / (ms / 1e3), "rows": rows,
                               "note": "includes one device copy of the windows (the reference's windowed H2D "
                                       "lands them in its work buffer)"}
    del x, work
    torch.cuda.empty_cache()
    # PWS (substack 1) on 256 pairs x 720 traces x 2001 lags; TF-PWS on 8 pairs
    npairs, ntr, n = 256, 720, 2001
    t = torch.randn((npairs * ntr, n), generator=g, device=dev, dtype=torch.float32)
    w = torch.full((npairs * ntr,), 1.0 / ntr, dtype=torch.float32, device=dev)
    lin = t.view(npairs, ntr, n).mean(dim=1)
    ms = _timed(torch, stream, lambda: ref_gpu.pws_run_device(t, w, [ntr] * npairs, lin), reps=2, warm=1)
    out["pws"] = {"ms": ms, "traces_per_s": npairs * ntr / (ms / 1e3), "pairs": npairs, "traces": ntr,
                  "nsamples": n, "power": 1.0}
    del t, w, lin
    torch.cuda.empty_cache()
    rng = np.random.default_rng(3)
    tp = 8
    pre = [sto.tfpws_prestack(rng.standard_normal((ntr, n)), 10) for _ in range(tp)]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for gr, wt, li in pre:
        ref_gpu.tfpws_run(gr.astype(np.float32), wt.astype(np.float32), li.astype(np.float32), 0.1,
                          band=(0.05, 5.0, -1.0))
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    out["tfpws"] = {"ms": ms, "pairs_per_s": tp / (ms / 1e3), "pairs": tp, "groups": len(pre[0][1]),
                    "wall_s": time.perf_counter() - t0,
                    "note": "per pair as the reference (one pair per compute call), 64-frequency chunks"}
    return out


def serving_run(args, device: int, rank: int) -> dict:
    """Poisson stream of correlation jobs (mean args.serve_rate per s for
    args.serve_seconds): subarrays of 2-200 stations from a 1000-station
    pool x 1-30 days, delta 0.05/0.1/0.2 s, lag 50-200 s, 10% with PWS;
    synthetic station-day spectra resident in HBM across jobs."""
    from fastxc_gb300.serve import Server, poisson_stream

    srv = Server(device=device, slots=args.serve_slots, cache_gib=48.0, work_gib=150.0, chunk_gib=6.0,
                 synthetic=True, seed=rank, max_wait_s=2.0, keep_results=True)
    try:
        # warm-up: geometry, FFT tables and pair plans of each delta
        for d in (0.05, 0.1, 0.2):
            jid = srv.submit(np.arange(4, dtype=np.int32), 0, 1, d, 100.0)
            srv.wait(jid, timeout_s=120.0)
            srv.release(jid)
        recs, wall, failures = poisson_stream(srv, args.serve_seconds, args.serve_rate, seed=100 + rank,
                                              wait_limit_s=args.serve_wait_limit)
        st = srv.stats()
    finally:
        srv.close()
    lat = np.array([r["latency"] for r in recs]) if recs else np.zeros(1)
    qw = np.array([r["queue"] for r in recs]) if recs else np.zeros(1)
    svc = lat - qw  # start -> results in host memory, queueing excluded
    pwin = float(sum(r["pair_windows"] for r in recs))
    return {"jobs": len(recs), "arrival_rate_per_s": args.serve_rate, "arrival_seconds": args.serve_seconds,
            "slots": args.serve_slots, "p50_latency_s": float(np.percentile(lat, 50)),
            "p99_latency_s": float(np.percentile(lat, 99)), "mean_queue_s": float(qw.mean()),
            "p50_service_s": float(np.percentile(svc, 50)), "p99_service_s": float(np.percentile(svc, 99)),
            "mean_service_s": float(svc.mean()),
            # service seconds offered per slot-second of the arrival window:
            # above 1 the stream outruns the slots and latency is queueing
            "offered_load": float(svc.sum() / max(args.serve_seconds * args.serve_slots, 1e-9)),
            "max_latency_s": float(lat.max()), "pair_windows": pwin,
            "pair_windows_per_s": pwin / wall if wall > 0 else None, "makespan_s": wall,
            "pws_jobs": int(sum(r["pws"] for r in recs)), "cache_entries_end": int(st.cache_entries),
            "failed_jobs": len(failures), "failures": failures[:3],
            "latency": "submit -> NCFs (and PWS) in host memory, steady clock",
            "workload": "jobs: 2-200 of 1000 stations x 1-30 days, delta 0.05/0.1/0.2 s, lag 50-200 s, "
                        "10% PWS; win 3600 s; synthetic seeded spectra cached in HBM"}


def _rel(got, ref) -> float:
    """Largest per-row relative L2 error."""
    got = np.asarray(got).reshape(-1, np.asarray(got).shape[-1])
    ref = np.asarray(ref).reshape(-1, np.asarray(ref).shape[-1])
    return float((np.linalg.norm(got - ref, axis=1) / np.maximum(np.linalg.norm(ref, axis=1), 1e-30)).max())


def _timed(torch, stream, fn, reps=3, warm=1):
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def stages_run(torch, dev, local: int, hbm_gbs: float, fp32_tflops: float, stack_pairs: int = 2304,
               batch_block: int = 0, method_arg: str = "auto", batch_days: int = 10) -> dict:
    """The other stages of the path on their own configurations, timed with
    CUDA events on the launching stream (inputs resident, larger than L2):
      sac2spec: one day of 64 stations x 3 components at 10 Hz (192 rows x
        864 000 samples, 24 one-hour windows, RAM + whitening after);
      linear stack / PWS: 256 station pairs x 9 components, 720 NCF
        windows of 2001 lags each (13.3 GB), PWS power 2;
      TF-PWS: all of those pairs, substacks of 10 (72 groups), 0.05-5 Hz;
    each with its largest relative L2 error against the FP64 oracle on a
    sample of its inputs."""
    from fastxc_gb300 import sac2spec as s2s
    from fastxc_gb300 import stack
    from fastxc_gb300.core import Context

    out = {}
    stream = torch.cuda.current_stream(dev)
    ctx = Context(local, stream.cuda_stream)
    g = torch.Generator(device=dev)
    g.manual_seed(7)
    try:
        # --- sac2spec -------------------------------------------------------
        F = s2s.read_filter_file(ROOT / "tests" / "golden" / "filter_d0.1_0.1-2.txt")
        plan = s2s.plan(86400, 3600, 3600, 100, 0.1, F, s2s.WHITEN_AFTER, s2s.NORM_RUNABS)
        resp = torch.from_numpy(s2s.filter_response(plan, F)).to(dev)
        rows, npts = 192, plan.npts
        series = torch.randn((rows, npts), generator=g, device=dev, dtype=torch.float32)
        steps = np.arange(plan.nstep, dtype=np.int32)
        spec = torch.empty((plan.nstep, rows, plan.nspec), dtype=torch.complex64, device=dev)
        ms = _timed(torch, stream, lambda: s2s.run(ctx, plan, series, npts, npts, rows, 3, steps, resp, spec,
                                                   plan.nspec))
        units = rows * plan.nstep
        alg = units * (plan.segment_pts * 4 + plan.nspec * 8)
        out["sac2spec"] = {"channel_windows_per_s": units / (ms / 1e3), "ms": ms,
                           "workload": f"{rows} rows x {npts} samples, {plan.nstep} windows of {plan.segment_pts}, "
                                       f"nspec {plan.nspec}, RAM + whiten after",
                           "algorithmic_bytes": alg, "hbm_frac": alg / (ms / 1e3) / 1e9 / hbm_gbs,
                           "note": "algorithmic bytes = window read + spectrum write; FFT-bound"}
        from oracle import sac2spec_oracle as so

        op = so.make_plan(86400, 3600, 3600, 100, 0.1, so.read_filter_file(
            ROOT / "tests" / "golden" / "filter_d0.1_0.1-2.txt"), so.WHITEN_AFTER, so.NORM_RUNABS)
        sample_steps = [0, 11]
        wins = so.windows(series[:3].cpu().numpy().astype(np.float64), op, sample_steps)
        ref = so.run_rows(wins, op, 3)
        got = spec[sample_steps][:, :3].cpu().numpy()
        out["sac2spec"]["rel_l2_vs_fp64"] = _rel(got.reshape(-1, plan.nspec), ref.reshape(-1, plan.nspec))
        out["sac2spec"]["rel_l2_sample"] = "one station (3 channels) x windows 0 and 11, FP64 oracle"
        del series, spec, resp
        torch.cuda.empty_cache()
        # --- linear stack + PWS (config 3) ----------------------------------
        npairs, ntr, n = stack_pairs, 720, 2001
        t = torch.randn((npairs * ntr, n), generator=g, device=dev, dtype=torch.float32)
        offs = np.arange(npairs, dtype=np.int64) * ntr
        cnts = np.full(npairs, ntr, np.int32)
        lin = torch.empty((npairs, n), dtype=torch.float32, device=dev)
        ms = _timed(torch, stream, lambda: stack.linear_stack(ctx, t, offs, cnts, n, lin))
        nbytes = t.numel() * 4 + lin.numel() * 4
        out["linear_stack"] = {"traces_per_s": npairs * ntr / (ms / 1e3), "ms": ms, "bytes": nbytes,
                               "hbm_gbs": nbytes / (ms / 1e3) / 1e9, "hbm_frac": nbytes / (ms / 1e3) / 1e9 / hbm_gbs,
                               "workload": f"{npairs} pairs x {ntr} traces x {n} lags (sums bit-identical to FP64 accumulation)"}
        res = {}

        def pws_once():
            d_g, d_w, d_l, goff, gcnt = stack.prestack(ctx, torch, t, offs, cnts, n, 1, stack.MODE_PWS)
            stack.pws(ctx, d_g, d_w, goff, gcnt, d_l, n, lin, 2.0)
            res["g"] = d_g

        ms = _timed(torch, stream, pws_once, reps=2)
        lin_pws = lin[:2].cpu().numpy()
        nbytes = t.numel() * 4 * 3 + lin.numel() * 4  # traces read, groups written and read, stack written
        out["pws"] = {"traces_per_s": npairs * ntr / (ms / 1e3), "ms": ms, "power": 2.0,
                      "hbm_gbs_algorithmic": nbytes / (ms / 1e3) / 1e9,
                      "hbm_frac": nbytes / (ms / 1e3) / 1e9 / hbm_gbs,
                      "workload": f"{npairs} pairs x {ntr} traces x {n} lags, substack 1 (prestack + PWS)"}
        res.clear()
        # --- TF-PWS: every pair ----------------------------------------------------
        d_g, d_w, d_l, goff, gcnt = stack.prestack(ctx, torch, t, offs, cnts, n, 10, stack.MODE_TFPWS)
        o = torch.empty((npairs, n), dtype=torch.float32, device=dev)
        ms = _timed(torch, stream, lambda: stack.tfpws(ctx, d_g, d_w, goff, gcnt, d_l, n, o, 0.1, band=(0.05, 5.0)),
                    reps=1, warm=1)
        ng = int(gcnt[0])
        # S-transform work: (G + 1) inverse transforms of n per (pair, frequency)
        flops = npairs * (ng + 1) * (n // 2 + 1) * 5.0 * n * np.log2(n)
        out["tfpws"] = {"pairs_per_s": npairs / (ms / 1e3), "ms": ms, "groups": ng, "pairs": npairs,
                        "fft_flops": flops, "tflops": flops / (ms / 1e3) / 1e12,
                        "fp32_frac": flops / (ms / 1e3) / 1e12 / fp32_tflops,
                        "workload": f"{npairs} pairs x {ntr} traces -> {ng} groups of 10, {n} lags, 0.05-5 Hz band"}
        # errors against the FP64 oracle on a sample of the stage inputs
        from oracle import stack_oracle as sto

        th = t[: 2 * ntr].cpu().numpy().reshape(2, ntr, n)
        e_pws = [_rel(lin_pws[p], sto.pws(th[p], 1, 2.0)) for p in range(2)]
        e_tf = _rel(o[0].cpu().numpy(), sto.tfpws(th[0], 10, 1.0, band=(0.05, 5.0), delta=0.1))
        out["pws"]["rel_l2_vs_fp64"] = max(e_pws)
        out["pws"]["rel_l2_sample"] = "2 pairs x 720 traces, FP64 oracle"
        out["tfpws"]["rel_l2_vs_fp64"] = e_tf
        out["tfpws"]["rel_l2_sample"] = "1 pair x 720 traces, FP64 oracle"
        del t, lin, d_g, d_w, d_l, o
        torch.cuda.empty_cache()
        out["batching"] = batching_run(torch, dev, ctx, stream, batch_block, method_arg, batch_days)
        out["plain_small"] = small_run(torch, dev, ctx)
    finally:
        ctx.close()
    return out


def small_run(torch, dev, ctx) -> dict:
    """The small plain configuration end to end through the host-buffer
    call (pinned spectra in, NCFs out): 4 stations x 3 components, one day
    of 24 windows, nspec 18523, the 6 station pairs x 9 components."""
    from fastxc_gb300.core import PairPlan, xc_shape
    from fastxc_gb300.synthetic import cross_station_pairs

    nsta, nstep, nspec = 4, 24, 18523
    nchan = 3 * nsta
    src, rec = cross_station_pairs(nsta)
    rng = np.random.default_rng(1)
    h = torch.empty((nstep, nchan, nspec), dtype=torch.complex64, pin_memory=True)
    h.copy_(torch.from_numpy((rng.standard_normal((nstep, nchan, nspec)) +
                              1j * rng.standard_normal((nstep, nchan, nspec))).astype(np.complex64)))
    shape = xc_shape(nspec, nstep, 0.1, 100.0)
    plan = PairPlan(ctx, src, rec, nchan)
    o = torch.empty((src.size, shape.cc_size), dtype=torch.float32, pin_memory=True)
    hs, ho = h.numpy(), o.numpy()
    times = []
    for i in range(6):
        t0 = time.perf_counter()
        ctx.xc_run_host(plan, hs, nstep, nchan, nspec, None, 1.0 / nstep, shape, ho, 0)
        if i > 0:
            times.append((time.perf_counter() - t0) * 1e3)
    ms = statistics.median(times)
    return {"ms": ms, "pair_windows": int(src.size * nstep), "pair_windows_per_s": src.size * nstep / (ms / 1e3),
            "method": "plain", "workload": f"{nsta} sta x 3 comp, 1 day = {nstep} windows, nspec {nspec}, "
                                          f"{src.size} pairs, host buffers in and out (median of 5)"}


def batching_run(torch, dev, ctx, stream, block: int = 0, method_arg: str = "auto", days: int = 10) -> dict:
    """The batching configuration: 500 stations x 3 components at seeded
    positions in a 400 x 400 km square, split at random into a 3600-s and an
    1800-s window group (the reference runs each group separately: their
    spectra differ in length); per group the component pairs of its station
    pairs within 150 km; `days` days, each station-day covering a contiguous
    run of U(10%, 100%) of the day's windows at a random offset (the rest
    masked), so window counts per pair are uneven. One step = every day of
    both groups: per group-day the pack, one persistent contraction launch
    (or the plain stack) and the finalize. The method is autotuned on each
    group's first day unless method_arg names it. Rate = covered
    pair-windows (windows that both stations of a pair hold) / time."""
    from fastxc_gb300 import sac2spec as s2s
    from fastxc_gb300._lib import FXC_XC_PLAIN, FXC_XC_TENSOR
    from fastxc_gb300.core import Context, PairPlan, xc_shape

    rng = np.random.default_rng(4)
    nsta = 500
    pos = rng.uniform(0.0, 400.0, (nsta, 2))
    in_3600 = rng.random(nsta) < 0.5
    F = s2s.read_filter_file(ROOT / "tests" / "golden" / "filter_d0.1_0.1-2.txt")
    g = torch.Generator(device=dev)
    g.manual_seed(11)
    groups = []
    for win, sel in ((3600, np.nonzero(in_3600)[0]), (1800, np.nonzero(~in_3600)[0])):
        plan = s2s.plan(86400, win, win, 100, 0.1, F, s2s.WHITEN_AFTER, s2s.NORM_RUNABS)
        nstep, nspec, n = int(plan.nstep), int(plan.nspec), sel.size
        nchan = 3 * n
        p = pos[sel]
        dist = np.hypot(p[:, None, 0] - p[None, :, 0], p[:, None, 1] - p[None, :, 1])
        si, sj = np.nonzero(np.triu(dist <= 150.0, 1))
        a, b = np.meshgrid(np.arange(3), np.arange(3), indexing="ij")
        src = (3 * si[:, None] + a.reshape(1, -1)).reshape(-1).astype(np.int32)
        rec = (3 * sj[:, None] + b.reshape(1, -1)).reshape(-1).astype(np.int32)
        # per station-day coverage: a contiguous run of U(10%, 100%) of the windows
        cnt = np.maximum(1, np.round(rng.uniform(0.1, 1.0, (days, n)) * nstep).astype(np.int64))
        off = (rng.random((days, n)) * (nstep - cnt + 1)).astype(np.int64)
        w = np.arange(nstep)
        sta_mask = ((w[None, :, None] >= off[:, None, :]) & (w[None, :, None] < (off + cnt)[:, None, :]))
        mask = np.repeat(sta_mask, 3, axis=2).astype(np.uint8)  # [day][win][chan]
        lo = np.maximum(off[:, si], off[:, sj])
        hi = np.minimum(off[:, si] + cnt[:, si], off[:, sj] + cnt[:, sj])
        covered = int(np.maximum(hi - lo, 0).sum()) * 9
        spec = torch.randn((days, nstep, nchan, nspec), generator=g, device=dev, dtype=torch.complex64)
        d_mask = torch.from_numpy(mask).to(dev)
        shape = xc_shape(nspec, nstep, 0.1, 100.0)
        pitch = (nspec + 3) // 4 * 4
        pl = PairPlan(ctx, src, rec, nchan)
        method, layout, tune_ms = ctx.xc_autotune_layout(pl, spec[0], nstep, nchan, nspec, nspec)
        if method_arg != "auto":
            method = FXC_XC_TENSOR if method_arg == "tensor" else FXC_XC_PLAIN
        packed = None
        if method == FXC_XC_TENSOR:
            packed = torch.empty((Context.xc_packed_bytes(nchan, nstep, nspec) // 16, 4), dtype=torch.int32,
                                 device=dev)
        groups.append(dict(win=win, nsta=n, nchan=nchan, nstep=nstep, nspec=nspec, src=src, rec=rec,
                           station_pairs=int(si.size), covered=covered, spec=spec, mask=d_mask, shape=shape,
                           pitch=pitch, plan=pl, method=method,
                           autotune_ms=dict(tune_ms, layout=LAYOUT_NAMES.get(layout, layout)),
                           packed=packed,
                           stack=torch.empty((src.size, pitch), dtype=torch.complex64, device=dev),
                           ncf=torch.empty((src.size, shape.cc_size), dtype=torch.float32, device=dev)))

    def group_day(gr, d, c=ctx):
        scale = 1.0 / gr["nstep"]
        sp, mk = gr["spec"][d], gr["mask"][d]
        if gr["packed"] is not None:
            c.xc_pack(sp, gr["nstep"], gr["nchan"], gr["nspec"], gr["nspec"], mk, gr["packed"])
            c.xc_stack_packed(gr["plan"], gr["packed"], gr["nstep"], gr["nspec"], scale, gr["stack"], gr["pitch"])
        else:
            c.xc_stack(gr["plan"], sp, gr["nstep"], gr["nchan"], gr["nspec"], gr["nspec"], mk, scale, gr["stack"],
                       gr["pitch"], gr["method"])
        c.xc_finalize(gr["stack"], gr["src"].size, gr["pitch"], gr["shape"], gr["ncf"])

    def step(c=ctx):
        for gr in groups:
            for d in range(days):
                group_day(gr, d, c)

    ms = _timed(torch, stream, step, reps=2, warm=1)
    # the same step recorded once as a CUDA graph on a stream of its own
    # (one uncaptured run there sizes that context's scratch) and replayed
    gstream = torch.cuda.Stream(dev)
    gctx = Context(dev.index if dev.index is not None else 0, gstream.cuda_stream)
    graph_ms = None
    try:
        step(gctx)
        gstream.synchronize()
        gctx.graph_begin()
        step(gctx)
        graph = gctx.graph_end()
        graph_ms = _timed(torch, gstream, graph.launch, reps=2, warm=1)
        graph.close()
    finally:
        gctx.close()
    per_group = []
    for gr in groups:
        gms = _timed(torch, stream, lambda: [group_day(gr, d) for d in range(days)], reps=1, warm=0)
        per_group.append({"win_len_s": gr["win"], "stations": gr["nsta"], "station_pairs": gr["station_pairs"],
                          "pairs": int(gr["src"].size), "windows_per_day": gr["nstep"], "nspec": gr["nspec"],
                          "method": "tensor" if gr["method"] == FXC_XC_TENSOR else "plain",
                          "autotune_sample_ms": gr["autotune_ms"], "ms_per_day": gms / days,
                          "covered_pair_windows": gr["covered"],
                          "nominal_pair_windows": int(gr["src"].size) * gr["nstep"] * days})
    covered = sum(gr["covered"] for gr in groups)
    nominal = sum(int(gr["src"].size) * gr["nstep"] * days for gr in groups)
    out = {"pair_windows_per_s": covered / (ms / 1e3), "rate_basis": "covered pair-windows (both stations hold the window)",
           "nominal_pair_windows_per_s": nominal / (ms / 1e3), "ms_per_step": ms, "graph_ms_per_step": graph_ms,
           "graph_launches_per_step": 3 * days * len(groups), "days": days,
           "covered_pair_windows": covered, "nominal_pair_windows": nominal, "groups": per_group,
           "workload": f"500 sta x 3 comp in a 400 km square, split into 3600-s and 1800-s window groups, pairs "
                       f"within 150 km per group, {days} days, coverage U(10%,100%) per station-day at a random "
                       "offset; per group-day: pack + contraction (or plain stack) + finalize"}
    for gr in groups:
        gr.clear()
    del groups
    torch.cuda.empty_cache()
    return out


def profile_traffic(kernel: str, workload: str):
    """DRAM bytes (read + write) of one launch of `kernel` on `workload`, from
    the ncu summaries committed under profiles/ (their 'machine-readable'
    lines); None when no capture of that workload exists."""
    for p in sorted((ROOT / "profiles").glob("*.md")):
        for ln in p.read_text().splitlines():
            if ln.startswith("machine-readable:"):
                try:
                    d = json.loads(ln.split(":", 1)[1])
                except ValueError:
                    continue
                if d.get("kernel") == kernel and d.get("workload") == workload:
                    return int(d["traffic_bytes_per_launch"])
    return None


def profile_case(name: str) -> None:
    """Small cases of the non-xc stages for ncu captures: sac2spec on one
    day of 64 stations x 3 components, 4 windows (768 rows), run twice;
    stacking: PWS on 64 pairs x 720 traces x 2001 lags (substack 1) and
    TF-PWS on 8 of them (substacks of 10, 0.05-5 Hz)."""
    import torch

    import __graft_entry__

    __graft_entry__.build()
    from fastxc_gb300 import sac2spec as s2s
    from fastxc_gb300 import stack
    from fastxc_gb300.core import Context

    dev = torch.device("cuda", 0)
    g = torch.Generator(device=dev)
    g.manual_seed(1)
    with Context(0) as ctx:
        if name == "sac2spec":
            F = s2s.read_filter_file(ROOT / "tests" / "golden" / "filter_d0.1_0.1-2.txt")
            plan = s2s.plan(86400, 3600, 3600, 100, 0.1, F, s2s.WHITEN_AFTER, s2s.NORM_RUNABS)
            resp = torch.from_numpy(s2s.filter_response(plan, F)).to(dev)
            rows, npts = 192, plan.npts
            series = torch.randn((rows, npts), generator=g, device=dev, dtype=torch.float32)
            steps = np.arange(4, dtype=np.int32)
            spec = torch.empty((4, rows, plan.nspec), dtype=torch.complex64, device=dev)
            for _ in range(2):
                s2s.run(ctx, plan, series, npts, npts, rows, 3, steps, resp, spec, plan.nspec)
        else:
            npairs, ntr, n = 64, 720, 2001
            t = torch.randn((npairs * ntr, n), generator=g, device=dev, dtype=torch.float32)
            offs = np.arange(npairs, dtype=np.int64) * ntr
            cnts = np.full(npairs, ntr, np.int32)
            out = torch.empty((npairs, n), dtype=torch.float32, device=dev)
            dg, dw, dl, goff, gcnt = stack.prestack(ctx, torch, t, offs, cnts, n, 1, stack.MODE_PWS)
            stack.pws(ctx, dg, dw, goff, gcnt, dl, n, out, 2.0)
            dg, dw, dl, goff, gcnt = stack.prestack(ctx, torch, t[: 8 * ntr], offs[:8], cnts[:8], n, 10,
                                                    stack.MODE_TFPWS)
            o = torch.empty((8, n), dtype=torch.float32, device=dev)
            stack.tfpws(ctx, dg, dw, goff, gcnt, dl, n, o, 0.1, band=(0.05, 5.0))
        ctx.synchronize()
    print(f"profile case {name} done")


def main():
    args = parse()
    if args.profile_case:
        profile_case(args.profile_case)
        return
    if args.impl == "reference":
        run_reference(args)
        return
    import torch

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    import __graft_entry__

    __graft_entry__.build()
    from fastxc_gb300 import lib
    from fastxc_gb300._lib import FXC_XC_LAYOUT_WHOLE_BIN, FXC_XC_PLAIN, FXC_XC_TENSOR, FxcError
    from fastxc_gb300.core import Context, PairPlan, xc_shape
    from fastxc_gb300 import replicas
    from fastxc_gb300.synthetic import cross_station_pairs, spectra_device, station_array

    nspec = args.nspec
    nwin = NSTEP * args.days
    arr = station_array(NSTA, seed=0)
    nchan = arr.nchan
    src, rec = cross_station_pairs(NSTA)
    npairs = src.size
    stream = torch.cuda.current_stream(dev)
    ctx = Context(local, stream.cuda_stream)
    plan = PairPlan(ctx, src, rec, nchan)
    shape = xc_shape(nspec, NSTEP, DT, CC_LEN)
    # resident spectra rows padded to a multiple of 4 bins (32 bytes): the
    # fused contraction loads the 4 bins of a sector with two 16-byte loads
    spec_pitch = (nspec + 3) // 4 * 4
    spec_buf = torch.zeros((nwin, nchan, spec_pitch), dtype=torch.complex64, device=dev)
    spec, mask = spectra_device(torch, nwin, arr, nspec, DT, seed=rank, gap_frac=GAP_FRAC, device=dev,
                                out=spec_buf[:, :, :nspec])
    scale = 1.0 / nwin  # mean over days of per-day stacks with 1/nstep each
    spec_bytes = nwin * nchan * nspec * 8
    pitch_stack = (nspec + 3) // 4 * 4
    d_stack = torch.empty((npairs, pitch_stack), dtype=torch.complex64, device=dev)
    d_ncf = torch.empty((npairs, shape.cc_size), dtype=torch.float32, device=dev)
    torch.cuda.synchronize()

    methods = {"plain": FXC_XC_PLAIN}
    try:
        ctx.xc_stack(plan, spec, nwin, nchan, nspec, spec_pitch, None, scale, d_stack, pitch_stack, FXC_XC_TENSOR)
        torch.cuda.synchronize()
        methods["tensor"] = FXC_XC_TENSOR
    except FxcError:
        pass
    autotune = None
    if args.method == "auto":
        m, lay, ms = ctx.xc_autotune_layout(plan, spec, nwin, nchan, nspec, spec_pitch)
        head = "tensor" if m == FXC_XC_TENSOR and "tensor" in methods else "plain"
        autotune = {"method": head, "layout": LAYOUT_NAMES.get(lay, lay), "sample_bins": min(nspec, 512),
                    "sample_ms": ms}
    else:
        head = args.method
        if head not in methods:
            raise SystemExit(f"method {head} not available")

    packed_bytes = Context.xc_packed_bytes(nchan, nwin, nspec)
    d_packed = None

    # with FXC_GEMM_FUSED=1 the whole-bin layout reads the FP32 spectra
    # itself (the pack fused into the contraction); otherwise pack first
    fused = "tensor" in methods and plan.layouts(nwin)[1] == FXC_XC_LAYOUT_WHOLE_BIN and \
        os.environ.get("FXC_GEMM_FUSED") == "1"
    if "tensor" in methods and not fused:
        d_packed = torch.empty((max(packed_bytes, 16) // 16, 4), dtype=torch.int32, device=dev)

    def step(method, ev=None):
        # events: 0 start, 1 after pack (separate pack only), 2 after stack, 3 after finalize
        if ev is not None:
            ev[0].record(stream)
        if method == FXC_XC_TENSOR and fused:
            if ev is not None:
                ev[1].record(stream)
            ctx.xc_stack(plan, spec, nwin, nchan, nspec, spec_pitch, None, scale, d_stack, pitch_stack, method)
        elif method == FXC_XC_TENSOR:
            ctx.xc_pack(spec, nwin, nchan, nspec, spec_pitch, None, d_packed)
            if ev is not None:
                ev[1].record(stream)
            ctx.xc_stack_packed(plan, d_packed, nwin, nspec, scale, d_stack, pitch_stack)
        else:
            if ev is not None:
                ev[1].record(stream)
            ctx.xc_stack(plan, spec, nwin, nchan, nspec, spec_pitch, None, scale, d_stack, pitch_stack, method)
        if ev is not None:
            ev[2].record(stream)
        ctx.xc_finalize(d_stack, npairs, pitch_stack, shape, d_ncf)
        if ev is not None:
            ev[3].record(stream)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # the contraction kernel of the plan's layout: one CTA per bin over both
    # triangle tiles (whole bin, up to 192 channels) or persistent CTAs over
    # (tile, bin) items
    gemm_kernel = ("k_xc_tc_gemm_bin" if plan.layouts(nwin)[1] == FXC_XC_LAYOUT_WHOLE_BIN else "k_xc_tc_gemm")
    results = {}
    sampler = ClockSampler(local)
    clocks = None
    for name in (["plain", "tensor"] if "tensor" in methods else ["plain"]):
        m = methods[name]
        for _ in range(args.warmup):
            step(m)
        torch.cuda.synchronize()
        evs = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.steps)]
        barrier()
        torch.cuda.synchronize()
        if name == head:
            sampler.start()
        lib().fxc_launch_count_reset()
        ctx.kernel_timing(True)  # CUDA events around each contraction kernel launch
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        t_start.record(stream)
        for i in range(args.steps):
            step(m, evs[i])
        t_end.record(stream)
        torch.cuda.synchronize()
        launches = lib().fxc_launch_count()
        gemm_total, gemm_n = ctx.kernel_time(gemm_kernel)
        ctx.kernel_timing(False)
        barrier()
        if name == head:
            clocks = sampler.stop()
        total_ms = replicas.reduce_max(t_start.elapsed_time(t_end), device=dev)
        pack_ms = statistics.mean(e[0].elapsed_time(e[1]) for e in evs)
        kern_ms = statistics.mean(e[1].elapsed_time(e[2]) for e in evs)
        fin_ms = statistics.mean(e[2].elapsed_time(e[3]) for e in evs)
        ncf_snapshot = d_ncf[:16].float().cpu().numpy().copy()
        gemm_ms = gemm_total / gemm_n if gemm_n else None
        results[name] = {"total_ms": total_ms, "ms_per_step": total_ms / args.steps, "pack_ms": pack_ms,
                         "stack_ms": kern_ms, "finalize_ms": fin_ms, "launches": launches, "ncf16": ncf_snapshot,
                         "gemm_ms": gemm_ms}

    # one day (the first 24 windows) through fxc_xc_run: the unit the
    # reference's xc_fast processes per timestamp
    one_day = {}
    for name in results:
        d_ncf1 = torch.empty((npairs, shape.cc_size), dtype=torch.float32, device=dev)
        one_day[name] = _timed(torch, stream, lambda: ctx.xc_run(plan, spec[:NSTEP], NSTEP, nchan, spec_pitch, None,
                                                                  1.0 / NSTEP, shape, d_ncf1, methods[name]),
                               reps=3, warm=1)
        del d_ncf1
    one_day_line = {k: {"ms": v, "pair_windows_per_s": npairs * NSTEP / (v / 1e3)} for k, v in one_day.items()}
    one_day_line["workload"] = f"{npairs} pairs x {NSTEP} windows x nspec {nspec} (one day), fxc_xc_run"

    # parity sample: 16 pairs over all windows against the FP64 oracle
    from oracle import xc_oracle as xo

    sel = np.arange(16)
    chans = np.unique(np.concatenate([src[sel], rec[sel]]))
    remap = {c: i for i, c in enumerate(chans)}
    host_spec = spec[:, torch.tensor(chans, device=dev), :].cpu().numpy()
    oshape = xo.finalize_shape(nspec, NSTEP, DT, CC_LEN)
    ref = xo.xc_run(host_spec, np.array([remap[c] for c in src[sel]]), np.array([remap[c] for c in rec[sel]]),
                    scale, oshape)
    rel = {}
    for name, r in results.items():
        e = np.linalg.norm(r["ncf16"] - ref, axis=1) / np.linalg.norm(ref, axis=1)
        rel[name] = float(e.max())
    if "tensor" in results:
        a, b = results["tensor"]["ncf16"], results["plain"]["ncf16"]
        rel["tensor_vs_plain"] = float((np.linalg.norm(a - b, axis=1) / np.linalg.norm(b, axis=1)).max())

    pw = npairs * nwin
    hr = results[head]
    value = replicas.whole_job_rate(pw, world, hr["total_ms"] / args.steps / 1e3)

    # roofline of the dominant kernel: the tcgen05 GEMM (tensor) or the plain
    # stack kernel, each timed with CUDA events on the launching stream
    peaks = {}
    wkey = f"{nchan}ch_{nwin}win_nspec{nspec}"
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())
    useful_flop = 8.0 * nspec * pw  # one complex MAC (8 flop) per pair-window-bin
    if head == "tensor":
        # issued MMA flops: per (tile, bin, 32-window block) 24 MMAs of 128 x n x 16
        nkb = (nwin + 31) // 32
        sum_n = 0
        for a0 in range(0, nchan, 128):
            for b0 in range(a0, nchan, 256):
                sum_n += (min(256, nchan - b0) + 15) // 16 * 16
        issued = float(nspec) * nkb * 24 * 2 * 128 * 16 * sum_n
        # the contraction kernel's own launches, timed with CUDA events on
        # the context stream around each launch (fxc_ctx_kernel_timing); the
        # stack stage also holds the bin-major -> [pair][bin] transpose
        kms = hr["gemm_ms"] if hr.get("gemm_ms") else hr["stack_ms"]
        achieved = issued / (kms / 1e3) / 1e12
        # the burst peak applies when the sampled SM clock sat at its maximum
        # with no power cap during the timed region, the sustained one otherwise
        at_max = bool(clocks and clocks.get("sm_mhz") and clocks.get("sm_max_mhz")
                      and clocks["sm_mhz"] >= 0.95 * clocks["sm_max_mhz"]
                      and "sw_power_cap" not in (clocks.get("reasons") or []))
        if at_max and "bf16_tflops" in peaks:
            peak, peak_src = peaks["bf16_tflops"], "of measured burst bf16 (cuBLAS; clocks at max, no power cap)"
        elif "bf16_tflops_sustained" in peaks:
            peak, peak_src = peaks["bf16_tflops_sustained"], "of measured sustained bf16 (cuBLAS, power-capped clocks)"
        else:
            peak, peak_src = 1900.0, "of fallback 1.9 PFLOP/s burst"
        useful_tf = useful_flop / (kms / 1e3) / 1e12
        roofline = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                    "traffic": profile_traffic(gemm_kernel, wkey), "peak_source": peak_src, "kernel": gemm_kernel,
                    "algorithmic": "issued MMA flops = nspec x ceil(nwin/32) x 24 x (2 x 128 x 16 x n) summed over tiles "
                                   "(3 bf16 hi/lo products, Re and Im, upper-triangle tiles)",
                    "useful_tflops": useful_tf, "useful_x3_frac": 3.0 * useful_tf / peak,
                    "issued_over_useful_x3": issued / (3.0 * useful_flop), "kernel_ms": kms,
                    "stack_stage_ms": hr["stack_ms"], "pack_ms": hr["pack_ms"], "finalize_ms": hr["finalize_ms"],
                    "pack": "fused into the contraction (FP32 spectra read once)" if fused else "separate k_xc_pack"}
    else:
        kms = hr["stack_ms"]
        achieved = useful_flop / (kms / 1e3) / 1e12
        sm_max = peaks.get("sm_max_mhz", 2070.0)
        peak = 152 * 128 * 2 * sm_max * 1e6 / 1e12
        roofline = {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                    "traffic": profile_traffic("k_xc_stack_plain", wkey), "peak_source": "nominal FP32 (152 SMs x 128 lanes x 2 x max SM clock)",
                    "kernel": "k_xc_stack_plain", "algorithmic": "8 flop x nspec x pair-windows",
                    "kernel_ms": kms, "finalize_ms": hr["finalize_ms"]}

    line = {
        "metric": "pair-windows/s",
        "value": value,
        "unit": "pair-windows/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": hr["ms_per_step"],
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "bf16x3->f32" if head == "tensor" else "f32",
        "data": "synthetic (seeded whitened-like spectra, coherent 0.1-2 Hz source, 5% gap windows)",
        "method": head,
        "config": {"workload": f"xc linear stack: {NSTA} sta x {NCOMP} comp x {args.days} days, delta {DT}s, "
                               f"win 3600s -> {nwin} windows, nspec {nspec}, {npairs} pairs, lag {CC_LEN}s",
                   "pairs": npairs, "windows": nwin, "nspec": nspec, "cc_size": shape.cc_size,
                   "l2": f"inputs ({spec_bytes / 1e9:.1f} GB) larger than L2 (129 MB), no flush", "parallelism": f"replicas x{world}"},
        "rel_l2_vs_fp64": rel,
        "per_method": {k: {"pair_windows_per_s": pw / (v["ms_per_step"] / 1e3), "ms_per_step": v["ms_per_step"],
                           "pack_ms": v["pack_ms"], "stack_ms": v["stack_ms"], "finalize_ms": v["finalize_ms"],
                           **({"stack_kernel_fp32_frac": useful_flop / (v["stack_ms"] / 1e3) / 1e12 /
                               (152 * 128 * 2 * peaks.get("sm_max_mhz", 2070.0) * 1e6 / 1e12),
                               "fp32_peak": "nominal FP32 (152 SMs x 128 lanes x 2 x max SM clock)"}
                              if k == "plain" else {})}
                       for k, v in results.items()},
        "roofline": roofline,
        "one_day": one_day_line,
        "autotune": autotune,
        "gpu_launches": hr["launches"],
        "clocks": clocks,
    }
    if "tensor" in results:
        line["tensor_vs_plain_speedup"] = results["plain"]["ms_per_step"] / results["tensor"]["ms_per_step"]
        # the two kernels' own fractions beside the ratio: the plain stack
        # against the FP32 FMA peak (useful flops), the contraction against
        # the bf16 peak of its roofline (issued MMA flops)
        sm_max = peaks.get("sm_max_mhz", 2070.0)
        fp32_peak = 152 * 128 * 2 * sm_max * 1e6 / 1e12
        plain_tf = useful_flop / (results["plain"]["stack_ms"] / 1e3) / 1e12
        line["speedup_kernels"] = {"plain_stack_tflops": plain_tf, "plain_stack_fp32_frac": plain_tf / fp32_peak,
                                   "fp32_peak_tflops": fp32_peak,
                                   "contraction_bf16_frac": roofline["frac"] if head == "tensor" else None}

    # end-to-end through the host-buffer C-ABI call
    if not args.no_e2e:
        host_spec = torch.empty(spec.shape, dtype=torch.complex64, pin_memory=True)
        host_spec.copy_(spec)
        host_ncf = torch.empty((npairs, shape.cc_size), dtype=torch.float32, pin_memory=True)
        del d_stack, d_packed
        torch.cuda.empty_cache()
        hs = host_spec.numpy()
        hn = host_ncf.numpy()
        m = methods[head]
        ctx.xc_run_host(plan, hs, nwin, nchan, nspec, None, scale, shape, hn, m)
        barrier()
        e2e_steps = max(1, min(args.steps, 5))
        per_call = []
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            c0 = time.perf_counter()
            ctx.xc_run_host(plan, hs, nwin, nchan, nspec, None, scale, shape, hn, m)
            per_call.append((time.perf_counter() - c0) * 1e3)
        el = replicas.reduce_max((time.perf_counter() - t0) / e2e_steps, device=dev)
        # the floor: the same spectra copied over the host link in the
        # pipeline's 64-window chunks, back to back, with nothing else running
        # (the fastest of three: the host link's rate fluctuates on these boxes)
        copy_ms = float("inf")
        floor_buf = torch.empty((64, nchan, nspec), dtype=torch.complex64, device=dev)
        for _ in range(3):
            c0 = torch.cuda.Event(enable_timing=True)
            c1 = torch.cuda.Event(enable_timing=True)
            c0.record(stream)
            with torch.cuda.stream(stream):
                for w0 in range(0, nwin, 64):
                    nw = min(64, nwin - w0)
                    floor_buf[:nw].copy_(host_spec[w0:w0 + nw], non_blocking=True)
            c1.record(stream)
            torch.cuda.synchronize()
            copy_ms = min(copy_ms, c0.elapsed_time(c1))
        # three more calls with the phase record on (CUDA events on both
        # streams), each with its wall time: whether a slow call's time is
        # in its host-to-device copies or in the pipeline behind them
        ctx.kernel_timing(True)
        phase_calls = []
        for _ in range(3):
            c0 = time.perf_counter()
            ctx.xc_run_host(plan, hs, nwin, nchan, nspec, None, scale, shape, hn, m)
            wall = (time.perf_counter() - c0) * 1e3
            phase_calls.append(dict(ctx.host_phases(), wall=wall))
        ctx.kernel_timing(False)
        phases = phase_calls[0]
        line["e2e"] = {"value": replicas.whole_job_rate(pw, world, el), "unit": "pair-windows/s",
                       "h2d_bytes_per_step": int(spec.numel() * 8), "d2h_bytes_per_step": int(npairs * shape.cc_size * 4),
                       "ms_per_step": el * 1e3, "steps": e2e_steps,
                       "h2d_copy_ms": copy_ms, "h2d_gbs": spec.numel() * 8 / (copy_ms / 1e3) / 1e9,
                       "over_copy_floor": el * 1e3 / copy_ms, "ms_per_call": per_call,
                       "median_ms_per_call": float(np.median(per_call)), "phase_ms": phases,
                       "phase_calls": [{k: (round(v, 2) if isinstance(v, float) else v) for k, v in c.items()}
                                       for c in phase_calls],
                       "phase_note": "three extra calls with CUDA events on the copy and compute streams (phase_ms "
                                     "is the first): copy_busy = sum of H2D copy durations, compute_busy = sum of "
                                     "per-chunk compute, tail = time after the last H2D copy ends, wall = the "
                                     "call's host wall time"}

    # the step's buffers are released before the stage timings and the
    # serving stream (which uses its own HBM arenas)
    d_stack = d_packed = d_ncf = spec = spec_buf = mask = floor_buf = None
    host_spec = host_ncf = hs = hn = None
    plan = None
    ctx.close()
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    if not args.no_stages and world == 1:
        line["stages"] = stages_run(torch, dev, local, peaks.get("hbm_gbs", 6800.0),
                                    152 * 128 * 2 * peaks.get("sm_max_mhz", 2070.0) * 1e6 / 1e12,
                                    args.stack_pairs, args.batch_block, args.method, args.batch_days)
    if args.serve_seconds > 0:
        # serving: a Poisson stream of correlation jobs against the engine
        line["serving"] = serving_run(args, local, rank)

    if rank == 0 and world == 1 and not args.no_cpu:
        cores = os.cpu_count() or 1
        v, sample = cpu_baseline(seconds_target=12.0, threads=cores)
        line["cpu_baseline"] = {"value": v, "unit": "pair-windows/s", "cores": cores, "kind": "port", "sample": sample,
                                "cpu_model": cpu_model()}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
