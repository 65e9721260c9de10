"""Benchmark: fused F+X GSample/s on one GB300 (or N replicas), one JSON line.

Workload (default): 24 inputs, n_freq 16384 (32768-sample frames), 4096 frames
per integration -- the precision workload the throughput target is quoted on.
A step is one integration: zero the accumulator, F-engine + X-engine over all
4096 frames (passes of 1024 frames), scale by 1/4096. Inputs (3.2 GB of int8)
are generated in HBM before timing and are larger than L2, so no flush is needed.

  value      : device-resident throughput, int8 samples in per second (GS/s)
  e2e        : the same integration through the C ABI (corr_row_accumulate from
               the pinned staging ring, H2D inside the timed region, fetch to host)
  roofline   : the dominant kernel's achieved algorithmic bytes/s vs measured HBM
  cpu_baseline: the numpy float64 oracle (the reference's gen_golden.py
               formulation) on a bounded sample, on this host's cores
  batching   : 64 integration blocks of 512..8192 frames (24 inputs, n_freq 16384,
               0.5% packet loss, pooled 8192-frame ring) in one CUDA-graph launch:
               aggregate GS/s and per-block latency p50/p99
  stream     : 40 inputs, n_freq 16384, 4096-frame integrations with the split
               tensor X-engine: GS/s and the real-time factor against 40 x 250 MS/s

--impl reference runs the reference's CPU formulation of the path (the oracle
port, multi-process over all host cores) on the same workload and metric.
"""

from __future__ import annotations

import argparse
import importlib
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))
PKG_NAME = "21cma_abf_correlator_gb300"
METRIC = "fused F+X GSample/s"
PASS_FRAMES = 1024        # default frames per F/X pass on the device-resident path


def peaks():
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    return 6800.0, 1900.0, "fallback"


def sm_max_mhz() -> float:
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text()).get("sm_max_mhz", 2070.0))
    return 2070.0


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-i", str(self.gpu), "-lms", "100"], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_oracle_sample(w, frames: int, seed_offset: int = 0):
    synth = importlib.import_module(PKG_NAME + ".synth")
    x, mask = synth.generate_numpy(w, frames, seed_offset)
    present = None if mask is None else synth.unpack_mask(mask, frames)
    return x, present


def _oracle_worker(args):
    """Generate a sample (untimed), then time the oracle on it."""
    name, frames, seed_offset = args
    synth = importlib.import_module(PKG_NAME + ".synth")
    oracle = importlib.import_module("oracle.corr_oracle")
    w = synth.WORKLOADS[name]
    x, present = cpu_oracle_sample(w, frames, seed_offset)
    t0 = time.perf_counter()
    oracle.correlate(x, present)
    return time.perf_counter() - t0


def time_cpu_oracle(w, target_s: float, processes: int) -> dict:
    """Time the float64 oracle on frames of this workload, spread over `processes`."""
    L = w.fft_len
    # calibrate in this process: one warm call (first-call costs), then the
    # marginal cost per frame between 4 and 16 frames
    _oracle_worker((w.name, 1, 0))
    t4 = _oracle_worker((w.name, 4, 0))
    t16 = _oracle_worker((w.name, 16, 0))
    per_frame = max((t16 - t4) / 12, t16 / 32, 1e-4)
    frames_per_proc = max(1, int(target_s / per_frame))
    frames_per_proc = min(frames_per_proc, 512)
    if processes <= 1:
        wall = _oracle_worker((w.name, frames_per_proc, 1))
    else:
        import multiprocessing as mp
        ctx = mp.get_context("spawn")
        with ctx.Pool(processes) as pool:
            pool.map(_oracle_worker, [(w.name, 1, 100 + i) for i in range(processes)])  # warm
            # workers run concurrently; the slowest one's compute time is the wall
            wall = max(pool.map(_oracle_worker, [(w.name, frames_per_proc, 200 + i)
                                                 for i in range(processes)]))
    samples = w.n_station * frames_per_proc * processes * L
    return {"value": samples / wall / 1e9, "unit": "GSample/s", "cores": processes,
            "sample": f"{frames_per_proc * processes} frames x {w.n_station} inputs x {L} samples "
                      f"({w.name}), numpy float64 rfft + per-baseline sum, "
                      f"{processes} process(es) of one thread each (pocketfft, einsum), "
                      f"{wall:.1f} s wall"}


def run_reference(args) -> None:
    world, rank, _ = dist_env()
    if rank != 0:
        return
    synth = importlib.import_module(PKG_NAME + ".synth")
    w = synth.WORKLOADS[args.workload]
    procs = os.cpu_count() or 1
    vals = []
    for _ in range(args.warmup):
        time_cpu_oracle(w, min(3.0, args.cpu_seconds), procs)
    for _ in range(args.steps):
        vals.append(time_cpu_oracle(w, args.cpu_seconds, procs))
    v = statistics.median([x["value"] for x in vals])
    frames_step = w.frames
    samples_step = w.n_station * frames_step * w.fft_len
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "GSample/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": samples_step / (v * 1e9) * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": w.name, "n_station": w.n_station, "n_freq": w.n_freq,
                   "frames_per_integration": w.frames, "path": "numpy float64 oracle "
                   "(reference corr-cuda/tests/gen_golden.py formulation) on host cores"},
        "cpu_baseline": {"value": v, "unit": "GSample/s", "cores": procs, "kind": "port",
                         "sample": vals[-1]["sample"]},
        "e2e": {"value": v, "unit": "GSample/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main() -> None:
    global PASS_FRAMES
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="precision-24in-nf16384")
    ap.add_argument("--xmode", default="auto", choices=["auto", "plain", "tc", "tc_split"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--frames", type=int, default=0,
                    help="override frames per integration (smaller cases for profiling)")
    ap.add_argument("--pass-frames", type=int, default=PASS_FRAMES,
                    help="frames per F/X pass (spectra buffer depth)")
    ap.add_argument("--no-tune", action="store_true",
                    help="keep the default tile shapes instead of autotuning them")
    ap.add_argument("--tiles", default="",
                    help="XCT,XKT,FPLAN[,YTILE]: fixed tensor tile, FFT plan and spectra "
                         "layout (default n_freq) instead of the autotuner's (profiling a "
                         "chosen configuration)")
    ap.add_argument("--only", default="", choices=["", "frontend", "writer"],
                    help="run just one side workload (the synthetic front end or the file "
                         "writer) on this workload's geometry and print its JSON")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the error report against the float64 DFT")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the batching and stream workloads")
    args = ap.parse_args()
    PASS_FRAMES = args.pass_frames
    args.warmup = max(args.warmup, 3)

    if args.impl == "reference":
        run_reference(args)
        return
    if args.only:
        run_only(args)
        return

    import torch
    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    build = importlib.import_module(PKG_NAME + ".build")
    if rank == 0:
        build.build()
    if world > 1:
        torch.distributed.barrier()
    pkg = importlib.import_module(PKG_NAME)
    synth = importlib.import_module(PKG_NAME + ".synth")
    abi = pkg.abi
    w = synth.WORKLOADS[args.workload]
    if args.frames:
        import dataclasses
        w = dataclasses.replace(w, frames=args.frames)
    N, nf, F, L = w.n_station, w.n_freq, w.frames, w.fft_len
    B = w.n_baseline

    modes = {"plain": abi.CORR_X_PLAIN_FP32, "tc": abi.CORR_X_TC_FP16,
             "tc_split": abi.CORR_X_TC_FP16_SPLIT}
    if args.xmode == "auto":
        candidates = ["tc_split", "tc", "plain"]
    else:
        candidates = [args.xmode]
    # per-visibility error bound each path is tested to (vs the float64 oracle):
    # plain and split 1e-5 / 2e-5 at any length; FP16 6e-3/sqrt(frames)
    err_bound = {"plain": 1e-5, "tc_split": 2e-5, "tc": 6e-3 / math.sqrt(F)}

    x, mask = synth.generate_torch(
        w, F, seed_offset=importlib.import_module(PKG_NAME + ".replicas").replica_seed_offset(rank))
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    samples_step = N * F * L

    def make_step(eng, acc, row):
        # the integration accumulates in complex128 (FP64 cross-launch
        # accumulator) and is dumped, divided by its frame count, into a
        # complex64 row
        def step():
            acc.zero_()
            eng.accumulate(x, F, acc, mask=mask, stream=stream)
            eng.dump(acc, F, row, stream=stream)
        return step

    results = {}
    engines = {}
    tiles = {}
    for name in candidates:
        try:
            eng = pkg.FxEngine(N, nf, PASS_FRAMES, xmode=modes[name])
            if args.tiles:
                vals = [int(v) for v in args.tiles.split(",")]
                xct, xkt, fplan = vals[:3]
                eng.set_tiles(vals[3] if len(vals) > 3 else nf, xct, xkt, fplan)
                tiles[name] = eng.tiles()
            elif args.no_tune:
                tiles[name] = eng.tiles()
            else:
                tiles[name] = eng.autotune(stream)
            eng.set_accumulator(abi.CORRX_ACC_FP64)
            acc = eng.new_acc()
            row = torch.empty((B, nf), dtype=torch.complex64, device="cuda")
            step = make_step(eng, acc, row)
            step()
            torch.cuda.synchronize()
            eng.check()
        except pkg.CorrError as e:
            if e.status == abi.CORR_ERR_NOT_IMPL:
                continue
            raise
        engines[name] = (eng, acc, step, row)
    if not engines:
        raise SystemExit("no X-engine available")
    # FFT plan 2 (the tensor-core F-engine, n_freq 16384, FP16 spectra) on the FP16
    # path's tiles: reported beside the others, never the headline (it rounds the
    # data to FP16 between its DFT stages; the autotuner does not choose it)
    if "tc" in engines and nf == 16384 and not args.tiles:
        t_ = tiles["tc"]
        eng = pkg.FxEngine(N, nf, PASS_FRAMES, xmode=modes["tc"])
        eng.set_tiles(t_["ytile"], t_["xct"], t_["xkt"], 2)
        tiles["tc_tensor_fft"] = eng.tiles()
        eng.set_accumulator(abi.CORRX_ACC_FP64)
        acc = eng.new_acc()
        row = torch.empty((B, nf), dtype=torch.complex64, device="cuda")
        step = make_step(eng, acc, row)
        step()
        torch.cuda.synchronize()
        eng.check()
        engines["tc_tensor_fft"] = (eng, acc, step, row)
        err_bound["tc_tensor_fft"] = err_bound["tc"]

    def time_steps(step, k, w_):
        for _ in range(w_):
            step()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        return e0.elapsed_time(e1) / k

    # rows of each path for this integration (identical input every step), and
    # their errors against float64 over the whole row
    accuracy = None
    if rank == 0 and not args.no_accuracy:
        rows = {name: e_[3].clone() for name, e_ in engines.items()}
        accuracy = accuracy_report(torch, w, x, mask, rows)
        del rows
        torch.cuda.empty_cache()

    # the headline path: the fastest X-engine that meets the 1e-4 precision
    # target -- every visibility's error within 1e-4 of its two inputs' power
    # (and the row's rel. RMS within 1e-4) -- as measured over the whole row
    # against float64, or by its tested bound when no measurement was made
    def meets(name):
        if accuracy is not None and name in accuracy["vs_fp64_full_row"]:
            e = accuracy["vs_fp64_full_row"][name]
            return e["max_per_vis"] <= 1e-4 and e["rel_rms"] <= 1e-4
        return err_bound[name] <= 1e-4
    per_path = {}
    for name, e_ in engines.items():
        per_path[name] = time_steps(e_[2], 2, 1)
    eligible = [n for n in per_path if meets(n) and n != "tc_tensor_fft"] or list(per_path)
    best = min(eligible, key=per_path.get)
    eng, acc, step, row = engines[best]

    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    ms = time_steps(step, args.steps, args.warmup)
    clocks = sampler.stop()
    eng.check()

    replicas = importlib.import_module(PKG_NAME + ".replicas")
    ms = replicas.slowest_ms(ms, world, device="cuda")
    value = replicas.job_gsps(samples_step, world, ms)

    paths = {}
    for name, e_ in engines.items():
        m = ms if name == best else time_steps(e_[2], max(2, args.steps // 2), 1)
        paths[name] = {"value": samples_step / (m * 1e-3) / 1e9, "ms_per_step": m,
                       "tiles": {k: tiles[name][k] for k in ("ytile", "xct", "xkt", "fplan")},
                       "per_vis_err_bound": err_bound[name], "meets_1e-4": meets(name)}

    # what the FP64 cross-launch accumulator costs: the headline path with a
    # complex64 accumulator instead (scaled in place, no dump)
    acc32 = torch.zeros((B, nf), dtype=torch.complex64, device="cuda")
    eng.set_accumulator(abi.CORRX_ACC_FP32)

    def step32():
        acc32.zero_()
        eng.accumulate(x, F, acc32, mask=mask, stream=stream)
        eng.scale(acc32, F, stream=stream)
    ms32 = time_steps(step32, max(2, args.steps // 2), 1)
    eng.set_accumulator(abi.CORRX_ACC_FP64)
    del acc32
    accumulator = {"precision": "fp64 (complex128 row; each launch's FP32 sums added once)",
                   "ms_per_step_fp64": ms, "ms_per_step_fp32": ms32,
                   "cost_ms_per_integration": ms - ms32}

    # per-kernel times: one pass of PASS_FRAMES frames through each kernel alone
    hbm_peak, _, peak_kind = peaks()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    reps = 8
    for _ in range(2):
        abi.check(eng.lib.corrx_run_fengine(eng.h, x.data_ptr(), x.stride(0), x.stride(1),
                                            mask.data_ptr() if mask is not None else None,
                                            mask.stride(0) if mask is not None else 0, 0,
                                            PASS_FRAMES, stream.cuda_stream), "fengine")
        abi.check(eng.lib.corrx_run_xengine(eng.h, PASS_FRAMES, acc.data_ptr(),
                                            stream.cuda_stream), "xengine")
    torch.cuda.synchronize()
    t_f = t_x = 0.0
    for r in range(reps):
        f0 = (r * PASS_FRAMES) % (F - PASS_FRAMES + 1)
        base = x.data_ptr() + f0 * x.stride(1)
        ev[0].record(stream)
        abi.check(eng.lib.corrx_run_fengine(eng.h, base, x.stride(0), x.stride(1),
                                            mask.data_ptr() if mask is not None else None,
                                            mask.stride(0) if mask is not None else 0, f0,
                                            PASS_FRAMES, stream.cuda_stream), "fengine")
        ev[1].record(stream)
        abi.check(eng.lib.corrx_run_xengine(eng.h, PASS_FRAMES, acc.data_ptr(),
                                            stream.cuda_stream), "xengine")
        ev[2].record(stream)
        torch.cuda.synchronize()
        t_f += ev[0].elapsed_time(ev[1])
        t_x += ev[1].elapsed_time(ev[2])
    t_f /= reps
    t_x /= reps
    mb = synth.mask_bytes(F) if mask is not None else 0
    elem = 4 if best == "tc" else 8   # bytes per spectrum bin between the engines
    f_bytes = N * PASS_FRAMES * L + N * PASS_FRAMES * nf * elem + (N * mb * PASS_FRAMES // F)
    # spectra read once + the complex128 row read and written once per launch
    x_bytes = N * PASS_FRAMES * nf * elem + 2 * B * nf * 16
    # Nominal arithmetic of a length-L real FFT (half-length complex FFT + split):
    # 2.5 L log2 L flops. The FP32 peak is nominal (no measured figure on file):
    # SMs x 128 FMA lanes x 2 flops x the maximum SM clock.
    f_flops = 2.5 * L * math.log2(L) * N * PASS_FRAMES
    fp32_peak = (torch.cuda.get_device_properties(0).multi_processor_count * 128 * 2
                 * sm_max_mhz() * 1e6 / 1e12)
    kernels = {
        "fengine": {"ms_per_launch": t_f, "alg_bytes": f_bytes,
                    "achieved_gbs": f_bytes / (t_f * 1e-3) / 1e9,
                    "fp32": {"alg_flops": f_flops,
                             "alg_tflops": f_flops / (t_f * 1e-3) / 1e12,
                             "nominal_peak_tflops": fp32_peak,
                             "frac_of_nominal": f_flops / (t_f * 1e-3) / 1e12 / fp32_peak}},
        "xengine_" + best: {"ms_per_launch": t_x, "alg_bytes": x_bytes,
                            "achieved_gbs": x_bytes / (t_x * 1e-3) / 1e9,
                            "alg_tflops": 8.0 * B * nf * PASS_FRAMES / (t_x * 1e-3) / 1e12},
    }
    dom = "fengine" if t_f >= t_x else "xengine_" + best
    dk = kernels[dom]
    roofline = {"kernel": dom, "bound": "hbm", "achieved": dk["achieved_gbs"],
                "peak": hbm_peak, "unit": "GB/s", "frac": dk["achieved_gbs"] / hbm_peak,
                "peak_kind": peak_kind,
                "traffic": ncu_traffic(dom, w.name, PASS_FRAMES, best, paths[best]["tiles"]),
                "traffic_source": "profiles/traffic.json: ncu dram__bytes_read.sum + "
                                  "dram__bytes_write.sum of one captured launch, scaled to "
                                  "frames_per_launch",
                "alg_bytes_per_launch": dk["alg_bytes"], "frames_per_launch": PASS_FRAMES}
    if dom == "fengine":
        roofline["limiter"] = ("FP32 FFT arithmetic and shared-memory exchanges, not HBM: ncu on a "
                               "256-frame launch saw the FP32 pipe 52 % busy, shared-memory "
                               "wavefronts at 47 % and DRAM at 25 % of peak")

    e2e = None
    if not args.no_e2e and rank == 0:
        e2e = run_e2e(pkg, w, x, mask, modes[best], args, torch)

    extra = {}
    if not args.no_extra and rank == 0 and not args.frames:
        for e_ in engines.values():
            e_[0].close()
        del x, mask
        torch.cuda.empty_cache()
        # every block must meet 1e-4 at its own length: with the FP16 form as the
        # headline, blocks too short for its tested bound run on the split form
        if best == "tc":
            min_long = math.ceil((6e-3 / 1e-4) ** 2)          # 6e-3/sqrt(F) <= 1e-4
            extra["batching"] = run_batching(pkg, synth, torch, stream,
                                             [(modes["tc"], "tc", min_long),
                                              (modes["tc_split"], "tc_split", 0)])
        else:
            extra["batching"] = run_batching(pkg, synth, torch, stream,
                                             [(modes[best], best, 0)])
        torch.cuda.empty_cache()
        extra["stream"] = run_stream(pkg, synth, torch, stream)
        torch.cuda.empty_cache()
        extra["frontend"] = run_frontend(pkg, w, torch, stream)
        torch.cuda.empty_cache()
        extra["writer"] = run_writer(pkg, w)

    cpu = None
    if not args.no_cpu and rank == 0 and world == 1:
        # the reference's CPU formulation on every host core, as the reference arm
        # runs it: one short warm-up round, then the measured one
        procs = os.cpu_count() or 1
        time_cpu_oracle(w, min(3.0, args.cpu_seconds), procs)
        cpu = time_cpu_oracle(w, args.cpu_seconds, procs)
        cpu["kind"] = "port"

    passes = math.ceil(F / PASS_FRAMES)
    launches_per_step = 2 * passes + 1
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "GSample/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int8 in, f32 FFT, " + ("f32 X" if best == "plain" else "f16 tensor X"),
            "data": "synthetic (seeded Gaussian + common signal, delays; generated in HBM)",
            "config": {"workload": w.name, "n_station": N, "n_freq": nf,
                       "frames_per_integration": F, "baselines": B, "xengine": best,
                       "tiles": paths[best]["tiles"],
                       "frames_per_pass": PASS_FRAMES, "parallelism": f"replicas x{world}",
                       "l2": f"inputs {N * F * L / 1e9:.2f} GB per step > L2; no flush"},
            "paths": paths, "kernels": kernels, "roofline": roofline, "accuracy": accuracy,
            "accumulator": accumulator,
            "e2e": e2e, "cpu_baseline": cpu, "clocks": clocks,
            "gpu_launches": launches_per_step * args.steps,
        }
        line.update(extra)
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def ncu_traffic(kernel: str, workload: str, frames: int, path: str, tiles: dict):
    """DRAM bytes per launch of `kernel` on this workload and path, from the ncu
    captures summarised in profiles/traffic.json: bytes_per_frame * frames +
    bytes_per_launch (the F-engine's traffic is all per frame -- int8 read,
    spectra written; the X-engines' is the spectra read per frame plus the row's
    read and write per launch). None when no capture matches the configuration."""
    p = REPO / "profiles" / "traffic.json"
    if not p.exists():
        return None
    kind = "fengine" if kernel == "fengine" else "xengine"
    for e in json.loads(p.read_text()).get("captures", []):
        if (e["workload"] == workload and e["kernel"] == kind and e["path"] == path
                and e.get("fplan", 0) == tiles.get("fplan", 0)):
            return e["bytes_per_frame"] * frames + e["bytes_per_launch"]
    return None


def run_batching(pkg, synth, torch, stream, forms) -> dict:
    """64 uneven integration blocks captured in one CUDA graph (corrx_batch_*).

    forms: [(xmode, name, min_frames), ...] in order of preference; each block
    runs on the first form whose min_frames it reaches (one engine per form,
    corrx_batch_create_mixed when there are several). The packet loss is applied
    twice: at frame granularity (a frame with a lost packet is zeroed whole, the
    reference's receive rule; the main figures) and at packet granularity (only
    the lost 1024-sample packets are zeroed, corrx_batch_create_packets)."""
    import ctypes as C
    abi = pkg.abi
    w = synth.WORKLOADS["batching-24in-nf16384"]
    pool, mask, words = synth.generate_torch(w, w.frames, words=True)   # 8192-frame ring
    plan = synth.block_plan(w)
    nblk = len(plan)
    engs = []
    for xmode, _, _ in forms:
        e_ = pkg.FxEngine(w.n_station, w.n_freq, PASS_FRAMES, xmode=xmode)
        e_.autotune(stream)
        e_.set_accumulator(abi.CORRX_ACC_FP64)   # each block integrates in complex128
        engs.append(e_)
    which = [next(i for i, f in enumerate(forms) if b[1] >= f[2]) for b in plan]
    rows = torch.empty((nblk, w.n_baseline, w.n_freq), dtype=torch.complex64, device="cuda")
    host = torch.empty((nblk, w.n_baseline, w.n_freq), dtype=torch.complex64).pin_memory()
    first = (C.c_int64 * nblk)(*[b[0] for b in plan])
    frames = (C.c_int32 * nblk)(*[b[1] for b in plan])
    sel = (C.c_int32 * nblk)(*which)
    handles = (C.c_void_p * len(engs))(*[e_.h.value for e_ in engs])
    lib = engs[0].lib
    total_frames = sum(b[1] for b in plan)
    samples = w.n_station * total_frames * w.fft_len

    def timed(packets: bool) -> dict:
        h = C.c_void_p()
        common = (C.c_void_p(pool.data_ptr()), pool.stride(0), pool.stride(1))
        if packets:
            abi.check(lib.corrx_batch_create_packets(
                handles, len(engs), sel, *common, None, 0, C.c_void_p(words.data_ptr()),
                words.stride(0), first, frames, nblk, C.c_void_p(rows.data_ptr()),
                C.c_void_p(host.data_ptr()), C.byref(h)), "corrx_batch_create_packets")
        else:
            abi.check(lib.corrx_batch_create_mixed(
                handles, len(engs), sel, *common, C.c_void_p(mask.data_ptr()), mask.stride(0),
                first, frames, nblk, C.c_void_p(rows.data_ptr()), C.c_void_p(host.data_ptr()),
                C.byref(h)), "corrx_batch_create_mixed")
        try:
            abi.check(lib.corrx_batch_launch(h, C.c_void_p(stream.cuda_stream)), "launch")
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            abi.check(lib.corrx_batch_launch(h, C.c_void_p(stream.cuda_stream)), "launch")
            e1.record(stream)
            torch.cuda.synchronize()
            for e_ in engs:
                e_.check()
            ms = e0.elapsed_time(e1)
            lat = (C.c_float * nblk)()
            abi.check(lib.corrx_batch_block_ms(h, lat, nblk), "corrx_batch_block_ms")
        finally:
            lib.corrx_batch_destroy(h)
        lat = np.array(list(lat))
        return {"value": samples / (ms * 1e-3) / 1e9, "ms_per_launch": ms,
                "latency_ms": {"p50": float(np.percentile(lat, 50)),
                               "p99": float(np.percentile(lat, 99)),
                               "max": float(lat.max())}}

    try:
        by_frame = timed(False)
        by_packet = timed(True)
    finally:
        for e_ in engs:
            e_.close()
    n_lost = int(((words.to(torch.int64) & 0xFFFFFFFF) != 0xFFFFFFFF).sum())
    return {"workload": w.name, "blocks": nblk, "frames_total": total_frames,
            "value": by_frame["value"], "unit": "GSample/s",
            "ms_per_launch": by_frame["ms_per_launch"], "graph_launches": 1,
            "latency_ms": by_frame["latency_ms"],
            "latency": "block start to its row in pinned host memory, inside the graph",
            "loss": f"{w.loss:.3%} of 1024-sample packets; frame-granular zero-fill (a frame "
                    f"with a lost packet is zeroed whole): {n_lost} of {words.numel()} "
                    f"pool frames",
            "packet_granular": dict(by_packet, loss="only the lost packets zero-filled "
                                                    "(corrx_batch_create_packets)"),
            "xengine": {f[1]: {"blocks": which.count(i), "min_frames": f[2]}
                        for i, f in enumerate(forms)}}


def run_stream(pkg, synth, torch, stream) -> dict:
    """40 inputs at 250 MS/s each: one 4096-frame integration with the split engine."""
    w = synth.WORKLOADS["stream-40in-nf16384"]
    x, mask, words = synth.generate_torch(w, w.frames, words=True)
    eng = pkg.FxEngine(w.n_station, w.n_freq, PASS_FRAMES,
                       xmode=pkg.abi.CORR_X_TC_FP16_SPLIT)
    tiles = eng.autotune(stream)
    eng.set_accumulator(pkg.abi.CORRX_ACC_FP64)
    acc = eng.new_acc()
    row = torch.empty((w.n_baseline, w.n_freq), dtype=torch.complex64, device="cuda")

    def step():
        acc.zero_()
        eng.accumulate(x, w.frames, acc, mask=mask, stream=stream)
        eng.dump(acc, w.frames, row, stream=stream)
    for _ in range(2):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(2):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    eng.check()
    ms = e0.elapsed_time(e1) / 2
    # error of the first integration against the float64 DFT at 16 channels
    acc_rep = accuracy_report(torch, w, x, mask, {"tc_split": row.clone()})
    # a 60-s stream's worth of integrations back to back (the input frames are a
    # resident pool reused per integration), each timed from its first launch
    # until its row is in pinned host memory
    n_int = math.ceil(60.0 * 250e6 / (w.frames * w.fft_len))
    host_row = torch.empty(row.shape, dtype=row.dtype, pin_memory=True)
    marks = [torch.cuda.Event(enable_timing=True) for _ in range(n_int + 1)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(n_int)]
    marks[0].record(stream)
    for i in range(n_int):
        if i:
            marks[i].record(stream)
        step()
        with torch.cuda.stream(stream):
            host_row.copy_(row, non_blocking=True)
        ends[i].record(stream)
    marks[n_int].record(stream)
    torch.cuda.synchronize()
    lat = sorted(marks[i].elapsed_time(ends[i]) for i in range(n_int))
    total_ms = marks[0].elapsed_time(marks[n_int])
    # the same integration with only the lost packets zero-filled
    wd = words.contiguous()

    def step_packets():
        acc.zero_()
        eng.accumulate(x, w.frames, acc, stream=stream, packets=wd)
        eng.dump(acc, w.frames, row, stream=stream)
    step_packets()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(2):
        step_packets()
    e1.record(stream)
    torch.cuda.synchronize()
    eng.check()
    ms_pk = e0.elapsed_time(e1) / 2
    acc_pk = accuracy_report(torch, w, x, None, {"tc_split": row.clone()}, words=wd)
    # the F-engine alone on one pass: algorithmic HBM bytes / time
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    lib = eng.lib
    for r in range(4):
        ev[0].record(stream)
        pkg.abi.check(lib.corrx_run_fengine(eng.h, x.data_ptr(), x.stride(0), x.stride(1),
                                            mask.data_ptr() if mask is not None else None,
                                            mask.stride(0) if mask is not None else 0, 0,
                                            PASS_FRAMES, stream.cuda_stream), "fengine")
        ev[1].record(stream)
        torch.cuda.synchronize()
    t_f = ev[0].elapsed_time(ev[1])
    f_bytes = w.n_station * PASS_FRAMES * (w.fft_len + w.n_freq * 8)
    hbm, _, kind = peaks()
    eng.close()
    gs = w.n_station * w.frames * w.fft_len / (ms * 1e-3) / 1e9
    need = w.n_station * 0.25
    return {"workload": w.name, "xengine": "tc_split", "value": gs, "unit": "GSample/s",
            "tiles": {k: tiles[k] for k in ("ytile", "xct", "xkt", "fplan")},
            "ms_per_integration": ms, "real_time_factor": gs / need,
            "real_time_need_gsps": need,
            "integrations_per_60s": 60.0 * 250e6 / (w.frames * w.fft_len),
            "sixty_seconds": {
                "integrations": n_int, "ms_total": total_ms,
                "gsps": w.n_station * w.frames * w.fft_len * n_int / (total_ms * 1e-3) / 1e9,
                "real_time_factor": 60e3 / total_ms * (n_int * w.frames * w.fft_len
                                                       / (60.0 * 250e6)),
                "latency_ms": {"p50": lat[len(lat) // 2],
                               "p99": lat[min(len(lat) - 1, math.ceil(0.99 * len(lat)) - 1)],
                               "max": lat[-1]},
                "latency": "first launch of the integration to its row in pinned host memory "
                           "(F+X, scale, device-to-host copy), CUDA events on one stream"},
            "fengine": {"ms_per_launch": t_f, "frames_per_launch": PASS_FRAMES,
                        "achieved_gbs": f_bytes / (t_f * 1e-3) / 1e9,
                        "frac_of_hbm": f_bytes / (t_f * 1e-3) / 1e9 / hbm, "peak_kind": kind},
            "accuracy_first_integration": {"channels": acc_rep["channels"],
                                           "baselines": acc_rep["baselines"],
                                           "vs_fp64": acc_rep["vs_fp64"]["tc_split"],
                                           "vs_fp64_full_row":
                                               acc_rep["vs_fp64_full_row"]["tc_split"]},
            "loss": f"{w.loss:.3%} of 1024-sample packets; frame-granular zero-fill (a frame "
                    f"with a lost packet is zeroed whole, the reference's rule)",
            "packet_granular": {
                "value": w.n_station * w.frames * w.fft_len / (ms_pk * 1e-3) / 1e9,
                "ms_per_integration": ms_pk,
                "real_time_factor": w.n_station * w.frames * w.fft_len / (ms_pk * 1e-3) / 1e9
                / need,
                "loss": "only the lost packets zero-filled (corrx_accumulate_packets)",
                "accuracy_first_integration_vs_fp64": acc_pk["vs_fp64"]["tc_split"],
                "accuracy_first_integration_vs_fp64_full_row":
                    acc_pk["vs_fp64_full_row"]["tc_split"]}}


ACCURACY_CHANNELS = [0, 1, 2, 63, 1234, 2047, 3000, 4096, 5555, 8191, 8192, 9000, 12345,
                     16000, 16382, 16383]


def accuracy_report(torch, w, x, mask, rows: dict, channels=ACCURACY_CHANNELS,
                    words=None) -> dict:
    """Errors of each path's rows for one integration (already divided by frames).

    vs_fp64: against an exact float64 DFT of every frame at `channels` (all
    baselines; lost frames zeroed as the engines do, and with `words` the lost
    1024-sample packets), computed on the device in float64 with matrix
    products of the int8 frames and the DFT columns.
    vs_plain: each tensor form against the plain FP32 path over the whole row.
    rel_rms = ||V - V_ref|| / ||V_ref||; max_per_vis = max |V - V_ref| /
    sqrt(|V_jj V_kk|) (the error relative to the two inputs' powers);
    elementwise_max / _rms = |V - V_ref| / |V_ref| over the visibilities with
    |V_ref| > 1e-3 sqrt(|V_jj V_kk|) (near-zero cross terms excluded).
    """
    N, F, L = w.n_station, w.frames, w.fft_len
    ch = [c for c in channels if c < w.n_freq]
    dev = x.device
    t = torch.arange(L, dtype=torch.float64, device=dev)
    ang = -2.0 * math.pi * torch.outer(t, torch.tensor(ch, dtype=torch.float64, device=dev)) / L
    Wm = torch.cat([torch.cos(ang), torch.sin(ang)], dim=1)          # [L, 2C]
    C_ = len(ch)
    Y = torch.empty((N, F, C_), dtype=torch.complex128, device=dev)
    step = 512
    for s_ in range(N):
        for f0 in range(0, F, step):
            blk = x[s_, f0:f0 + step].to(torch.float64)
            if mask is not None:
                fr = torch.arange(f0, min(f0 + step, F), device=dev)
                bits = (mask[s_, fr // 8].to(torch.int64) >> (fr % 8)) & 1
                blk = blk * bits.to(torch.float64)[:, None]
            if words is not None:
                P = L // 1024
                wd = words[s_, f0:f0 + step].to(torch.int64)[:, None]
                keep = (wd >> torch.arange(P, device=dev)) & 1                  # [f, P]
                blk = (blk.view(-1, P, 1024) * keep.to(torch.float64)[:, :, None]).view(-1, L)
            prod = blk @ Wm
            Y[s_, f0:f0 + step] = torch.complex(prod[:, :C_], prod[:, C_:])
    pairs = [(j, k) for j in range(N) for k in range(j, N)]
    jj = torch.tensor([p[0] for p in pairs], device=dev)
    kk = torch.tensor([p[1] for p in pairs], device=dev)
    ref = torch.einsum("bfc,bfc->bc", Y[jj], Y[kk].conj()) / F              # [B, C]
    auto_idx = torch.tensor([pairs.index((i, i)) for i in range(N)], device=dev)

    def errs(got, want):
        d = (got - want).abs()
        rel_rms = float(torch.linalg.vector_norm(got - want) / torch.linalg.vector_norm(want))
        autos = want[auto_idx].real.abs()                                    # [N, C]
        norm = torch.sqrt(autos[jj] * autos[kk])
        # elementwise relative error where the visibility is not near zero
        big = want.abs() > 1e-3 * norm
        rel = d[big] / want.abs()[big]
        return {"rel_rms": rel_rms, "max_per_vis": float((d / norm).max()),
                "elementwise_max": float(rel.max()),
                "elementwise_rms": float(torch.sqrt((rel ** 2).mean())),
                "elementwise_count": int(big.sum())}

    chi = torch.tensor(ch, device=dev)
    out = {"channels": ch, "baselines": len(pairs), "frames": F, "vs_fp64": {}, "vs_plain": {},
           "vs_fp64_full_row": {}}
    for name, r in rows.items():
        out["vs_fp64"][name] = errs(r[:, chi].to(torch.complex128), ref)
    del Y, ref
    # every visibility of the row against a float64 reference: float64 FFT of
    # every frame (cuFFT through torch, a comparator only) and float64 sums
    full = full_row_reference(torch, w, x, mask, words, jj, kk)
    for name, r in rows.items():
        out["vs_fp64_full_row"][name] = errs(r.to(torch.complex128), full)
    out["full_row_reference"] = ("float64 rfft of every frame (torch.fft) and float64 "
                                 "per-channel sums over all frames, every baseline and channel")
    del full
    if "plain" in rows:
        p_ = rows["plain"].to(torch.complex128)
        for name, r in rows.items():
            if name != "plain":
                out["vs_plain"][name] = errs(r.to(torch.complex128), p_)
    return out


def full_row_reference(torch, w, x, mask, words, jj, kk, step: int = 128):
    """complex128 [n_baseline, n_freq]: the integration's rows in float64."""
    N, F, L, nf = w.n_station, w.frames, w.fft_len, w.n_freq
    dev = x.device
    G = torch.zeros((nf, N, N), dtype=torch.complex128, device=dev)
    for f0 in range(0, F, step):
        blk = x[:, f0:f0 + step].to(torch.float64)                       # [N, f, L]
        f1 = f0 + blk.shape[1]
        if mask is not None:
            fr = torch.arange(f0, f1, device=dev)
            bits = (mask[:, fr // 8].to(torch.int64) >> (fr % 8)) & 1     # [N, f]
            blk *= bits.to(torch.float64)[:, :, None]
        if words is not None:
            P = L // 1024
            wd = words[:, f0:f1].to(torch.int64)[:, :, None]
            keep = ((wd >> torch.arange(P, device=dev)) & 1).to(torch.float64)   # [N, f, P]
            blk = (blk.view(N, -1, P, 1024) * keep[..., None]).view(N, -1, L)
        Y = torch.fft.rfft(blk, dim=-1)[..., :nf].permute(2, 0, 1)         # [nf, N, f]
        del blk
        G += Y @ Y.conj().transpose(1, 2)
        del Y
    return (G[:, jj, kk] / F).T.contiguous()


def run_only(args) -> None:
    """One side workload alone (for profiling it): --only frontend | writer."""
    import dataclasses
    pkg = importlib.import_module(PKG_NAME)
    importlib.import_module(PKG_NAME + ".build").build()
    synth = importlib.import_module(PKG_NAME + ".synth")
    w = synth.WORKLOADS[args.workload]
    if args.frames:
        w = dataclasses.replace(w, frames=args.frames)
    if args.only == "writer":
        print(json.dumps({"writer": run_writer(pkg, w)}), flush=True)
        return
    import torch
    torch.cuda.set_device(0)
    print(json.dumps({"frontend": run_frontend(pkg, w, torch, torch.cuda.current_stream())}),
          flush=True)


def run_frontend(pkg, w, torch, stream) -> dict:
    """The on-device synthetic front end (corrx_frontend_fill) writing one whole
    integration of this workload (frames + validity mask) into HBM, per pattern:
    samples generated per second and the write bandwidth against the measured peak."""
    fe = importlib.import_module(PKG_NAME + ".frontend")
    N, nf, F, L = w.n_station, w.n_freq, w.frames, w.fft_len
    x = torch.empty((N, F, L), dtype=torch.int8, device="cuda")
    m = torch.empty((N, (F + 7) // 8), dtype=torch.uint8, device="cuda")
    hbm, _, kind = peaks()
    out = {"workload": w.name, "frames": F, "unit": "GSample/s", "patterns": {}}
    for pattern in ("prng", "counter"):
        spec = fe.ReplaySpec(pattern=pattern, drop_rate=0.001, delay_stride=1)
        frame0 = spec.first_full_frame(nf)
        for _ in range(2):
            fe.fill(spec, nf, frame0, x, m, stream=stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(3):
            fe.fill(spec, nf, frame0, x, m, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / 3
        nbytes = x.numel() + m.numel()
        gbs = nbytes / (ms * 1e-3) / 1e9
        out["patterns"][pattern] = {"ms": ms, "value": N * F * L / (ms * 1e-3) / 1e9,
                                    "write_gbs": gbs, "frac_of_hbm": gbs / hbm,
                                    "peak_kind": kind}
    out["value"] = out["patterns"]["prng"]["value"]
    del x, m
    return out


def run_writer(pkg, w, n_rows: int = 8) -> dict:
    """The native file-set writer on rows of this workload (n_baseline x n_freq
    complex64 each), into a RAM-backed directory when the host has one, with an
    fsync per row: rows per second against the row period of the real-time
    stream (frames x 2 n_freq samples at 250 MS/s)."""
    import shutil
    import tempfile
    wr = importlib.import_module(PKG_NAME + ".writer")
    base = "/dev/shm" if os.path.isdir("/dev/shm") else None
    d = tempfile.mkdtemp(prefix="corr-writer-", dir=base)
    try:
        rng = np.random.default_rng(0)
        rows = [rng.standard_normal((w.n_baseline, w.n_freq * 2)).astype(np.float32)
                .view(np.complex64) for _ in range(2)]
        names = [f"S{i:02d}" for i in range(w.n_station)]
        t0 = time.perf_counter()
        with wr.RowWriter(d, names, w.n_freq, w.frames, "bench", queue_rows=4,
                          queue_full="block", fsync_every_rows=1) as wt:
            for i in range(n_rows):
                wt.write_row(rows[i % 2], 1_790_000_000_000 + i, i, i * w.frames,
                             [w.frames] * w.n_station)
            wt.sync()
        dt = time.perf_counter() - t0
    finally:
        shutil.rmtree(d, ignore_errors=True)
    row_bytes = w.n_baseline * w.n_freq * 8
    period_ms = w.frames * w.fft_len / 250e6 * 1e3
    return {"rows": n_rows, "row_bytes": row_bytes, "ms_per_row": dt * 1e3 / n_rows,
            "write_mbs": row_bytes * n_rows / dt / 1e6, "dir": base or "tmp",
            "fsync_every_rows": 1, "real_time_row_period_ms": period_ms,
            "headroom": period_ms / (dt * 1e3 / n_rows)}


def run_e2e(pkg, w, x, mask, xmode, args, torch) -> dict:
    """The integration through the C ABI: staging -> H2D -> F+X -> row -> host."""
    N, L, F = w.n_station, w.fft_len, w.frames
    # 256-frame slots in an 8-slot ring, as the shipped configuration has them
    # (config/correlator.yaml: frames_per_slot 256, block_slots 8); fewer for short
    # integrations (the ring is filled once from the integration's own frames)
    fps = min(256, max(1, F // 2))
    block_slots = max(2, min(8, F // fps))
    cfg = pkg.make_config(N, w.n_freq, fps, fps, block_slots, 1)
    c = pkg.Correlator(cfg)
    c.set_xengine(xmode)
    tiles = c.autotune() if not args.no_tune else None
    # fill the ring once from the device-resident inputs (receive side's job)
    host = x[:, : fps * block_slots].cpu().numpy()
    for g in range(N):
        v = c.staging(g)
        v.samples[:] = host[g].reshape(block_slots, fps, L)
    out = np.empty(c.fetch_bytes() // 8, dtype=np.complex64)
    import ctypes as C
    pinned = [C.c_void_p(), C.c_void_p()]
    for buf in pinned:
        pkg.abi.check(c.lib.corr_host_alloc(out.nbytes, C.byref(buf)), "corr_host_alloc")
    rows = C.c_int32()
    seq = [0]
    done = pkg.abi.NOTIFY_FN(lambda _user: None)

    def integration(i, blocking):
        for f0 in range(0, F, fps):
            s = seq[0]
            if s >= block_slots:
                c.row_slot_free(s - block_slots)
            for g in range(N):
                c.staging(g).mask[s % block_slots, :] = 0xFF
            c.row_accumulate(s, min(fps, F - f0))
            seq[0] += 1
        c.row_end(F)
        if blocking:
            pkg.abi.check(c.lib.corr_rows_fetch(c.ctx, pinned[0], out.nbytes, C.byref(rows)),
                          "corr_rows_fetch")
        else:
            # the row's fetch is queued and the next integration's copies start
            # at once; two pinned buffers alternate
            pkg.abi.check(c.lib.corr_rows_fetch_submit(c.ctx, pinned[i % 2], out.nbytes,
                                                       C.byref(rows), done, None),
                          "corr_rows_fetch_submit")

    def wait_fetches():
        while c.lib.corr_rows_fetch_ready(c.ctx) == pkg.abi.CORR_ERR_BUSY:
            time.sleep(20e-6)

    # wall clock on the host: the median of five rounds, so that a hiccup or two
    # of the host's scheduler does not stand for the path
    k = max(2, args.steps // 2)
    medians = {}
    for blocking in (True, False):
        for i in range(2):
            integration(i, blocking)
        wait_fetches()
        rounds = []
        for _ in range(5):
            t0 = time.perf_counter()
            for i in range(k):
                integration(i, blocking)
            wait_fetches()     # the last row is in host memory
            rounds.append((time.perf_counter() - t0) / k)
        medians[blocking] = (statistics.median(rounds), rounds)
    dt, rounds = medians[False]
    for s in range(seq[0] - 1, max(seq[0] - block_slots, 0) - 1, -1):
        c.row_slot_free(s)
    for buf in pinned:
        c.lib.corr_host_free(buf)
    c.close()
    mb = (fps + 7) // 8
    h2d = N * F * L + N * mb * (F // fps)
    d2h = w.n_baseline * w.n_freq * 8
    return {"value": N * F * L / dt / 1e9, "unit": "GSample/s", "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h, "ms_per_step": dt * 1e3, "steps": k,
            "rounds_ms": [r * 1e3 for r in rounds],
            "path": "corr_row_accumulate/row_end/rows_fetch_submit from pinned staging: each "
                    "row's fetch overlaps the next integration's copies",
            "blocking_fetch": {"value": N * F * L / medians[True][0] / 1e9,
                               "ms_per_step": medians[True][0] * 1e3,
                               "path": "the same with corr_rows_fetch, one integration after "
                                       "the other"},
            "tiles": tiles}


if __name__ == "__main__":
    main()
