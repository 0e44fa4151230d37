#!/usr/bin/env python
"""Benchmark of the SAR backprojection (adjoint) operator on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--case config2]

One step = one backprojection x = A^H y of the 2048^2-pixel x 4096-pulse x 4096-sample workload
(upsample 8, linear interpolation): the fused range-profile upsampling kernel followed by the
tiled gather kernel, with y resident in HBM.  The metric is pixel-pulses per second.  The roofline
denominator comes from the arithmetic-pipe rates measured on the same GPU in the same run
(sar_measure_pipe_rates); the CPU-baseline leg also checks the GPU image against the FP64 oracle
on a 256^2 patch over all pulses.

Prints one JSON line (rank 0).  ``--impl reference`` times the reference algorithm on the host
cores instead: the C restatement in oracle/ in the reference's own nearest-bin arithmetic
(bit-identical to the reference kernel where that kernel can be compiled), on a bounded pulse
sample of the same workload, all host threads.
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

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "backproj pixel·pulses/s @2048²×4096; CGLS s to 1e-3 resid, learned vs plain"
UNIT = "px*pulse/s"
SEED = 20261203


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--case", default="config2")
    ap.add_argument("--interp", choices=["linear", "nearest_ref"], default="linear",
                    help="interpolation of the --case run (profiling other settings; the headline is linear)")
    ap.add_argument("--upsample", type=float, default=None, help="upsample ratio of the --case run (default: the case's)")
    ap.add_argument("--cpu-pulses", type=int, default=96, help="pulse sample of the CPU baseline")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-cgls", action="store_true", help="skip the learned-vs-plain CGLS timing")
    ap.add_argument("--no-settings", action="store_true",
                    help="skip the other-settings timings (turned, diagonal, the reference's defaults)")
    ap.add_argument("--cgls-scenes", type=int, default=8)
    ap.add_argument("--suite", choices=["cgls", "autofocus", "resample", "cphd", "pdhg", "settings", "unet"],
                    default=None, help="run one of the library's other workloads instead of the benchmark")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def reduce_max(value: float, world: int, device=None) -> float:
    """Max of a per-rank value over all ranks (the job's clock is its slowest rank)."""
    if world <= 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank: float, world: int, ms_max: float) -> float:
    """Whole-job units/s: every rank runs the full workload (replicas), timed by the slowest rank."""
    return world * units_per_rank / (ms_max * 1e-3)


def measured_peaks():
    path = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return {}


class ClockSampler:
    """nvidia-smi clock / throttle sampling in the background (200 ms period)."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.proc = None
        ident = None
        try:
            import torch
            props = torch.cuda.get_device_properties(device_index)
            bus = getattr(props, "pci_bus_id", None)
            dom = getattr(props, "pci_domain_id", None)
            dev = getattr(props, "pci_device_id", None)
            if bus is not None and dom is not None and dev is not None:
                ident = f"{dom:08X}:{bus:02X}:{dev:02X}.0"
        except Exception:
            pass
        cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"]
        if ident:
            cmd.insert(1, f"--id={ident}")
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for name, v in zip(names, parts[4:8]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(name)
        if not sm:
            return {"samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------- ours
def run_ours(args):
    import torch
    from sarsolver_gb300 import NumpySimpleSarOperator
    from sarsolver_gb300.scenes import add_noise, config_workload, reflectivity

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    aperture, scene, upsample, desc = config_workload(args.case)
    if args.upsample:
        upsample = args.upsample
    S, N, P = aperture.num_slow_times, aperture.num_freqs, scene.num_scatterers
    n = scene.grid_shape[2]
    op = NumpySimpleSarOperator(scene, aperture, upsample_ratio=upsample, interp=args.interp, device=dev)
    plan = op.plan
    x_true = reflectivity(n, 500, 8.0, SEED, device=dev)
    y = add_noise(plan.forward(x_true), 20.0, SEED + 1)
    x = torch.empty(P, dtype=torch.complex64, device=dev)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    # ---- device-resident timing
    for _ in range(args.warmup):
        plan.adjoint(y, out=x)
    barrier()
    plan.enable_stage_timing(True)
    sampler = ClockSampler(local)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        plan.adjoint(y, out=x)
    e1.record(stream)
    barrier()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1) / args.steps
    stage_ms, calls = plan.stage_times()
    plan.enable_stage_timing(False)
    ms = reduce_max(ms, world, dev)
    value = job_throughput(P * S, world, ms)
    flags = plan.device_flags()   # every bounded wait and window check of the timed calls
    if flags:
        raise RuntimeError(f"device check flags {flags:#x} raised during the timed backprojections")

    # ---- forward projection y = A x (same workload), device-resident, stage-timed
    y_out = torch.empty((S, N), dtype=torch.complex64, device=dev)
    for _ in range(args.warmup):
        plan.forward(x_true, out=y_out)
    barrier()
    plan.enable_stage_timing(True)
    e0.record(stream)
    for _ in range(args.steps):
        plan.forward(x_true, out=y_out)
    e1.record(stream)
    barrier()
    fwd_ms = e0.elapsed_time(e1) / args.steps
    fstage, fcalls = plan.stage_times()
    plan.enable_stage_timing(False)

    # ---- end to end through the public operator API, host buffers (pinned)
    y_host = y.cpu().pin_memory()
    x_host = torch.empty(P, dtype=torch.complex64).pin_memory()
    for _ in range(args.warmup):
        x_host.copy_(op.backproject(y_host), non_blocking=True)
    barrier()
    e0.record(stream)
    for _ in range(args.steps):
        x_host.copy_(op.backproject(y_host), non_blocking=True)
    e1.record(stream)
    barrier()
    e2e_ms = reduce_max(e0.elapsed_time(e1) / args.steps, world, dev)

    # ---- roofline of the gather kernel: 28 FP32 flops + 3 special-function ops per pixel-pulse
    # (canonical work: range 10 + 1 sqrt, bin 3, interpolation 6, phase 1 + sin + cos, MAC 8), on the
    # FP32 and SFU rates measured on this GPU now
    props = torch.cuda.get_device_properties(dev)
    peaks = measured_peaks()
    sm_max = float(peaks.get("sm_max_mhz", 0.0)) or float((clocks or {}).get("sm_max_mhz", 0.0)) or 2070.0
    rates = pipe_rates(dev)
    fp32_units = 2.0 * rates["ffma_per_clk_sm"] / 28.0
    sfu_units = rates["sfu_sincos_per_clk_sm"] / 3.0
    units_per_clk = min(fp32_units, sfu_units)
    bound = "fp32" if fp32_units <= sfu_units else "sfu"
    r_roof = props.multi_processor_count * sm_max * 1e6 * units_per_clk
    k2_ms = stage_ms[1] / max(calls, 1)
    fft_ms = stage_ms[0] / max(calls, 1)
    achieved = P * S / (k2_ms * 1e-3)
    traffic = read_profile_traffic("bp_grid_ws_pair")
    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64 (fp32 arithmetic; double-float fp32 pairs for range/phase)",
        "data": "synthetic, seeded: 500 point scatterers + Gaussian-filtered (sigma 8 px) clutter x complex "
                "speckle, forward-projected by this operator, complex white noise at 20 dB SNR",
        "config": {"workload": f"{args.case}: backprojection, {desc}, {args.interp.replace('_ref', '')} interpolation",
                   "pixels": P, "pulses": S, "samples": N, "upsample": upsample,
                   "l2": "inputs larger than L2 (phase history %.0f MB, stored range profiles %.0f MB)"
                         % (S * N * 8 / 1e6, S * plan.profile_length * (8 if plan.tile_window > 256 else 16) / 1e6),
                   "parallelism": "replicas (each GPU runs the whole workload)" if world > 1 else "single GPU"},
        "stages_ms": {"upsample_fft_side": fft_ms, "gather_kernel": k2_ms},
        "forward": {"value": P * S / (fwd_ms * 1e-3), "unit": UNIT, "ms_per_step": fwd_ms,
                    "stages_ms": {"accumulator_clear": fstage[0] / max(fcalls, 1),
                                  "scatter_kernel": fstage[1] / max(fcalls, 1),
                                  "downsample_fft_side": fstage[2] / max(fcalls, 1)},
                    "note": "y = A x on the same workload (fp_grid_ws_kernel + FFT downsampling), not the headline"},
        "roofline": {"bound": bound, "kernel": "bp_grid_ws_pair_kernel", "achieved": achieved, "peak": r_roof,
                     "unit": "px*pulse/s", "frac": achieved / r_roof, "traffic": traffic,
                     "traffic_source": "from profile: ncu dram__bytes_read.sum + dram__bytes_write.sum per "
                                       "full-size launch, profiles/bp_grid_ws_pair_kernel_config2.md",
                     "peak_basis": f"{props.multi_processor_count} SMs x {sm_max:.0f} MHz (sm_max_mhz of "
                                   f"MEASURED_PEAKS.json) x min(2 x {rates['ffma_per_clk_sm']:.1f} FFMA/clk/SM / 28 "
                                   f"FP32 flops, {rates['sfu_sincos_per_clk_sm']:.1f} sin+cos/clk/SM / 3 SFU ops) "
                                   "per px*pulse; pipe rates measured in this run (sar_measure_pipe_rates)",
                     "pipe_rates": rates},
        "device_flags": flags,
        "e2e": {"value": job_throughput(P * S, world, e2e_ms), "unit": UNIT, "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": S * N * 8, "d2h_bytes_per_step": P * 8,
                "api": "NumpySimpleSarOperator.backproject(pinned host complex64 tensor) -> pinned host copy"},
        # our kernels per backprojection: per FFT chunk the fused upsampling kernel, or the packing
        # and unpacking kernels around cuFFT; then the gather
        "gpu_launches": args.steps * ((1 if plan.fused_upsampling else 2)
                                      * ((S + plan_chunk(plan) - 1) // plan_chunk(plan)) + 1),
        "clocks": clocks,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(aperture, scene, upsample, y, args.cpu_pulses, steps=1)
        check = oracle_check(aperture, scene, upsample, y, x, args.interp)
        result["oracle_rel_l2"] = check["rel_l2"]
        result["cpu_baseline"]["oracle_check"] = check
        result["cpu_baseline"]["config1"] = config1_cpu_gpu(dev)
        result["cpu_baseline"]["config4_lsqr"] = config4_lsqr_reference()
    if rank == 0 and not args.no_cgls:
        result["cgls"] = learned_vs_plain(args.cgls_scenes)
    if rank == 0 and not args.no_settings and args.case == "config2" and args.interp == "linear" and not args.upsample:
        # the same image and collection under the other settings (not the metric): looking along y
        # and along the diagonal, and the reference's defaults (nearest_ref, upsample 128)
        rows = settings_workload(rows=(("config2_turned", "linear", 8.0, "auto"),
                                       ("config2_diagonal", "linear", 8.0, "auto"),
                                       ("config2", "nearest_ref", 128.0, "auto")), verbose=False)
        result["settings"] = [{k: r[k] for k in ("case", "interp", "upsample", "adjoint_ms", "forward_ms",
                                                 "gather_shear", "scatter_shear", "scatter_ring_half")}
                              | {"gather_kernel_ms": r["adjoint_stages_ms"][1],
                                 "scatter_kernel_ms": r["forward_stages_ms"][1]} for r in rows]
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(result))


def learned_vs_plain(scenes: int) -> dict:
    """Second half of the metric: wall time of CGLS to ||A^H (y - A x)|| / ||A^H y|| <= 1e-3, plain
    (from zero) vs learned (U-Net warm start, then CGLS), on held-out generated scenes of the
    learned-solver workload (512^2 image, 1024 pulses x 1024 samples, aperture 2-6 deg, SNR
    10-30 dB).  Each solve is timed whole, host clock with device synchronisation around it."""
    import torch
    from sarsolver_gb300.learned import SceneSource, compare
    from sarsolver_gb300.train_warmstart import DEFAULT_WEIGHTS, load_warm_start, summary

    if not os.path.exists(DEFAULT_WEIGHTS):
        return {"unavailable": "no trained warm-start weights at " + os.path.relpath(DEFAULT_WEIGHTS, HERE)}
    warm, cfg = load_warm_start(DEFAULT_WEIGHTS)
    src = SceneSource(cfg, seed=424242, continuous=True)
    compare(warm, src, 1)                       # warm-up: plans, cuFFT plans, module loads
    recs = compare(warm, src, scenes, repeats=2, truth=True)
    # component times on the last scene's plan: one operator pair and one U-Net inference
    plan, y, _, _, _ = src.sample()
    b = plan.adjoint(y)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    timings = {}
    for name, fn in (("forward_ms", lambda: plan.forward(b)), ("adjoint_ms", lambda: plan.adjoint(y)),
                     ("unet_inference_ms", lambda: warm.direction(b))):
        for _ in range(3):
            fn()
        e0.record()
        for _ in range(10):
            fn()
        e1.record()
        torch.cuda.synchronize()
        timings[name] = e0.elapsed_time(e1) / 10
    src.close()
    out = summary(recs)
    out["component_ms"] = timings
    out.update({"metric": "CGLS wall time to normal-equations residual 1e-3", "unit": "ms",
                "higher_is_better": False, "learned_over_plain_time": out["learned_ms"] / out["plain_ms"],
                "workload": f"{cfg.n}^2 at {cfg.spacing} m, {cfg.num_pulses} pulses x {cfg.num_freqs} samples, "
                            f"U={cfg.upsample:g}, aperture U[{cfg.aperture_min:g},{cfg.aperture_max:g}] deg, "
                            f"SNR U[{cfg.snr_min:g},{cfg.snr_max:g}] dB",
                "weights": os.path.relpath(DEFAULT_WEIGHTS, HERE)})
    return out


def pipe_rates(dev) -> dict:
    """Per-SM arithmetic-pipe rates of this GPU (sar_measure_pipe_rates, include/sargpu.h)."""
    import ctypes
    import torch
    from sarsolver_gb300 import _lib

    lib = _lib.load()
    r = _lib.SarPipeRates()
    with torch.cuda.device(dev):
        _lib.check(lib.sar_measure_pipe_rates(ctypes.byref(r), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)),
                   "sar_measure_pipe_rates")
    return {"sfu_sincos_per_clk_sm": r.sfu_sincos_per_clk_sm, "frnd_per_clk_sm": r.frnd_per_clk_sm,
            "ffma_per_clk_sm": r.ffma_per_clk_sm, "ffma2_lanes_per_clk_sm": r.ffma2_per_clk_sm,
            "sms": r.num_sms, "probe_sm_mhz": r.sm_mhz}


def plan_chunk(plan) -> int:
    # one FFT chunk covers all pulses for every configuration here (4 GiB of rows)
    return plan.num_slow_times


def read_profile_traffic(kernel: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, if one exists."""
    path = os.path.join(HERE, "profiles", f"{kernel}_kernel_config2.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("dram_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


# -------------------------------------------------------------- CPU legs
def cpu_baseline(aperture, scene, upsample, y, pulses, steps=1):
    """Time the oracle port (FP64 C restatement, all host threads) on a pulse sample."""
    import oracle

    oracle.build()
    threads = oracle.default_threads()
    S = aperture.num_slow_times
    sel = np.linspace(0, S - 1, pulses).round().astype(int)
    y_np = y.cpu().numpy()[sel] if hasattr(y, "cpu") else np.asarray(y)[sel]
    prob = oracle.Problem(aperture.transmitter_positions[sel], aperture.receiver_positions[sel],
                          aperture.stab_ref_posns[sel], scene.positions, aperture.centre_frequency,
                          aperture.sample_bandwidth, aperture.num_freqs, upsample_ratio=upsample)
    units = scene.num_scatterers * pulses
    secs = {}
    for mode in ("linear", "nearest_ref"):
        t0 = time.perf_counter()
        for _ in range(steps):
            oracle.adjoint(prob, y_np, mode, threads=threads)
        secs[mode] = (time.perf_counter() - t0) / steps
    dt = secs["linear"]
    return {"value": units / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "nearest_ref_value": units / secs["nearest_ref"],
            "sample": f"full {scene.num_scatterers}-pixel image x {pulses} of {S} pulses "
                      f"({units:.3g} px*pulses), FP64, linear interpolation (value; the GPU path's arithmetic) "
                      f"{dt:.2f} s and nearest_ref (nearest_ref_value; the reference kernel's arithmetic) "
                      f"{secs['nearest_ref']:.2f} s per sample"}


def oracle_check(aperture, scene, upsample, y, x_gpu, mode="linear"):
    """FP64-oracle error of the timed workload's GPU image: the exact 256^2-pixel patch at the
    scene centre over all pulses (CPU-baseline leg; the oracle only checks, it is not timed as ours)."""
    import oracle

    S, N = aperture.num_slow_times, aperture.num_freqs
    n = scene.grid_shape[2]
    j0 = i0 = n // 2 - 128
    patch = np.asarray(scene.positions).reshape(n, n, 3)[j0:j0 + 256, i0:i0 + 256].reshape(-1, 3)
    prob = oracle.Problem(aperture.transmitter_positions, aperture.receiver_positions, aperture.stab_ref_posns,
                          patch, aperture.centre_frequency, aperture.sample_bandwidth, N, upsample_ratio=upsample)
    t0 = time.perf_counter()
    ref = oracle.adjoint(prob, y.cpu().numpy(), mode, threads=oracle.default_threads())
    dt = time.perf_counter() - t0
    got = x_gpu.reshape(n, n)[j0:j0 + 256, i0:i0 + 256].reshape(-1).cpu().numpy().astype(np.complex128)
    err = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
    return {"rel_l2": err, "pixels": int(patch.shape[0]), "pulses": S, "oracle_seconds": dt,
            "what": f"GPU backprojection of the timed workload vs the FP64 oracle ({mode}), 256^2 patch at the "
                    "scene centre, all pulses; target 1e-5"}


def config1_cpu_gpu(dev) -> dict:
    """Configuration 1 (128 pulses x 512 samples, U=8, 256^2 at 0.5 m, 3 deg): full forward and
    backprojection on the host cores (the oracle port, FP64, reference nearest-bin arithmetic and
    linear) and on the GPU, with the FP64-oracle error of the GPU results."""
    import oracle
    import torch
    from sarsolver_gb300 import SarPlan
    from sarsolver_gb300.scenes import add_noise, config_workload, reflectivity

    aperture, scene, upsample, desc = config_workload("config1")
    S, N, P = aperture.num_slow_times, aperture.num_freqs, scene.num_scatterers
    x = reflectivity(scene.grid_shape[2], 20, 8.0, SEED + 7, device=dev, clutter_level=0.0)
    plan = SarPlan(scene, aperture, upsample_ratio=upsample, interp="linear", device=dev)
    y = add_noise(plan.forward(x), 20.0, SEED + 8)
    prob = oracle.Problem(aperture.transmitter_positions, aperture.receiver_positions, aperture.stab_ref_posns,
                          scene.positions, aperture.centre_frequency, aperture.sample_bandwidth, N,
                          upsample_ratio=upsample)
    threads = oracle.default_threads()
    xn, yn = x.cpu().numpy(), y.cpu().numpy()
    out = {"workload": desc, "cores": threads, "units": P * S}
    for mode in ("nearest_ref", "linear"):
        t0 = time.perf_counter()
        yf = oracle.forward(prob, xn, mode, threads=threads)
        t1 = time.perf_counter()
        xa = oracle.adjoint(prob, yn, mode, threads=threads)
        t2 = time.perf_counter()
        out[f"cpu_{mode}_forward_s"] = t1 - t0
        out[f"cpu_{mode}_adjoint_s"] = t2 - t1
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for name, fn in (("forward", lambda: plan.forward(x)), ("adjoint", lambda: plan.adjoint(y))):
        for _ in range(3):
            fn()
        e0.record()
        for _ in range(20):
            r = fn()
        e1.record()
        torch.cuda.synchronize()
        out[f"gpu_linear_{name}_ms"] = e0.elapsed_time(e1) / 20
    out["gpu_forward_rel_l2"] = float(np.linalg.norm(plan.forward(x).cpu().numpy() - yf) / np.linalg.norm(yf))
    out["gpu_adjoint_rel_l2"] = float(np.linalg.norm(plan.adjoint(y).cpu().numpy() - xa) / np.linalg.norm(xa))
    plan.close()
    return out


def config4_lsqr_reference(n: int = 128, pulses: int = 256) -> dict:
    """CPU reference point of the learned-solver configuration at reduced size: scipy lsqr on the
    oracle port's operator pair (FP64, linear, all host threads) to the normal-equations residual
    ||A^H (y - A x)|| / ||A^H y|| <= 1e-3, as the GPU CGLS stops."""
    import oracle
    from scipy.sparse.linalg import LinearOperator, lsqr
    from sarsolver_gb300.scenes import grid_scene, spotlight_aperture

    aperture = spotlight_aperture(pulses, pulses, 4.0)
    scene = grid_scene(n, 0.25)
    P, S, N = scene.num_scatterers, pulses, pulses
    prob = oracle.Problem(aperture.transmitter_positions, aperture.receiver_positions, aperture.stab_ref_posns,
                          scene.positions, aperture.centre_frequency, aperture.sample_bandwidth, N, upsample_ratio=8.0)
    threads = oracle.default_threads()
    rng = np.random.default_rng(SEED + 4)
    x_true = np.zeros(P, np.complex128)
    idx = rng.choice(P, 40, replace=False)
    x_true[idx] = rng.standard_normal(40) + 1j * rng.standard_normal(40)
    y = oracle.forward(prob, x_true, "linear", threads=threads).reshape(-1)
    noise = rng.standard_normal(y.size) + 1j * rng.standard_normal(y.size)
    y = y + noise * np.sqrt(np.mean(np.abs(y) ** 2) / 10 ** (20 / 10) / 2)
    op = LinearOperator((S * N, P), dtype=np.complex128,
                        matvec=lambda v: oracle.forward(prob, v, "linear", threads=threads).reshape(-1),
                        rmatvec=lambda v: oracle.adjoint(prob, v.reshape(S, N), "linear", threads=threads))
    ahy = np.linalg.norm(op.rmatvec(y))

    def normal_residual(x):
        return float(np.linalg.norm(op.rmatvec(y - op.matvec(x))) / ahy)

    # lsqr has no stopping rule on ||A^H r|| / ||A^H y||.  It is CGLS in exact arithmetic, so CGLS
    # (numpy, the GPU solver's recurrence and stopping rule) finds the iteration count, then lsqr
    # runs that many iterations (one more pair at a time while the rule does not hold yet)
    t0 = time.perf_counter()
    x = np.zeros(P, np.complex128)
    r = y.copy()
    s_ = op.rmatvec(r)
    p_ = s_.copy()
    gamma = np.vdot(s_, s_).real
    k = 0
    while np.sqrt(gamma) / ahy > 1e-3 and k < 200:
        q = op.matvec(p_)
        alpha = gamma / np.vdot(q, q).real
        x += alpha * p_
        r -= alpha * q
        s_ = op.rmatvec(r)
        g_new = np.vdot(s_, s_).real
        p_ = s_ + (g_new / gamma) * p_
        gamma = g_new
        k += 1
    t_cgls = time.perf_counter() - t0
    it = max(k, 1)
    while True:
        t0 = time.perf_counter()
        x = lsqr(op, y, atol=0.0, btol=0.0, conlim=0.0, iter_lim=it)[0]
        dt = time.perf_counter() - t0
        resid = normal_residual(x)
        if resid <= 1e-3 or it >= 200:
            break
        it += 1
    return {"workload": f"{n}^2 at 0.25 m, {pulses} pulses x {pulses} samples, U=8, 4 deg, 40 points, 20 dB "
                        "(reduced size)", "iterations": it, "normal_residual": resid, "seconds": dt,
            "cgls_iterations": k, "cgls_seconds": t_cgls, "cores": threads,
            "solver": "scipy.sparse.linalg.lsqr on the FP64 oracle port (linear); CGLS (numpy) beside it"}


def run_reference(args):
    """The reference's own CPU arithmetic for this path, on the host cores: the oracle port in the
    nearest-bin mode (the reference kernel's only mode, sarsolver_cxx.cpp:319-353; the port is
    bit-identical to it where the reference compiles), all host threads, on a pulse sample of the
    benchmark workload.  Its phase history is the sample's forward projection (oracle, FP64) of a
    seeded scene of the benchmark's statistics plus 20 dB noise."""
    rank, world, _ = dist_info()
    if rank != 0:
        return
    import oracle
    from sarsolver_gb300.scenes import config_workload

    oracle.build()
    aperture, scene, upsample, desc = config_workload(args.case)
    S, N, P = aperture.num_slow_times, aperture.num_freqs, scene.num_scatterers
    pulses = max(1, args.cpu_pulses // 2)
    threads = oracle.default_threads()
    rng = np.random.default_rng(SEED)
    sel = np.linspace(0, S - 1, pulses).round().astype(int)
    prob = oracle.Problem(aperture.transmitter_positions[sel], aperture.receiver_positions[sel],
                          aperture.stab_ref_posns[sel], scene.positions, aperture.centre_frequency,
                          aperture.sample_bandwidth, N, upsample_ratio=upsample)
    x = 0.3 * (rng.standard_normal(P) + 1j * rng.standard_normal(P)) / np.sqrt(2.0)
    pts = rng.choice(P, 500, replace=False)
    x[pts] += (rng.standard_normal(500) + 1j * rng.standard_normal(500)) / np.sqrt(2.0)
    y = oracle.forward(prob, x, "nearest_ref", threads=threads)
    y += np.sqrt(np.mean(np.abs(y) ** 2) / 100.0 / 2.0) * (rng.standard_normal(y.shape) + 1j * rng.standard_normal(y.shape))
    for _ in range(args.warmup):
        oracle.adjoint(prob, y, "nearest_ref", threads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.adjoint(prob, y, "nearest_ref", threads=threads)
    dt = (time.perf_counter() - t0) / args.steps
    value = P * pulses / dt
    sample = (f"full {P}-pixel image x {pulses} of {S} pulses per step ({P * pulses:.3g} px*pulses), FP64, "
              "nearest_ref (the reference kernel's arithmetic)")
    print(json.dumps({
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c128 (fp64)",
        "data": "synthetic, seeded: 500 point scatterers + complex Gaussian clutter, forward-projected by the "
                "oracle, 20 dB noise",
        "config": {"workload": f"{args.case}: backprojection, {desc}, CPU pulse sample, nearest-bin sampling "
                               "(the reference has no linear interpolation)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


# ------------------------------------------------------------------ suites
# Other workloads of the library, one JSON line each (``python bench.py --suite NAME``): CUDA-event
# times of one call after a warm-up call.  Profiles under profiles/ cite these commands.
#   cgls       plain and learned CGLS, 512^2 x 1024 x 1024
#   autofocus  sharpness + phase gradient, 1024^2 x 2048 x 2048
#   resample   8192 x 8192 phase history, factors 2 x 2
#   cphd       8192 x 8192 CI4 CPHD file -> device
#   pdhg       100 PDHG iterations, 512^2 x 1024 x 1024
#   settings   one backprojection + one forward projection at 2048^2 x 4096 x 4096 per interpolation
#              mode, upsample factor and collection direction (one line per setting)
#   unet       forward and backward passes of the warm-start U-Net at 512^2

def _suite_time(fn, warmup: int = 1):
    import torch

    for _ in range(warmup):
        fn()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    out = fn()
    e1.record()
    torch.cuda.synchronize()
    return out, e0.elapsed_time(e1)


def cgls_workload() -> dict:
    import torch

    from sarsolver_gb300.learned import LearnedConfig, SceneSource
    from sarsolver_gb300.solvers import cgls
    from sarsolver_gb300.train_warmstart import DEFAULT_WEIGHTS, load_warm_start

    warm, cfg = load_warm_start(DEFAULT_WEIGHTS)
    src = SceneSource(cfg if isinstance(cfg, LearnedConfig) else LearnedConfig(), seed=31337, continuous=True)
    plan, y, _, extent, snr = src.sample()
    (_, plain), t_plain = _suite_time(lambda: cgls(plan, y, tol=1e-3, max_iterations=500))
    (_, learned), t_learned = _suite_time(lambda: warm.solve(plan, y, tol=1e-3, max_iterations=500))
    return {"workload": "cgls", "extent_deg": extent, "snr_db": snr, "plain_ms": t_plain,
            "plain_iterations": plain.iterations, "learned_ms": t_learned, "learned_iterations": learned.iterations}


def autofocus_workload() -> dict:
    import torch

    from sarsolver_gb300.autodiff import phase_weights, sharpness_gradient
    from sarsolver_gb300.plan import SarPlan
    from sarsolver_gb300.scenes import config_workload, reflectivity

    aperture, scene, upsample, _ = config_workload("config3")
    plan = SarPlan(scene, aperture, upsample_ratio=upsample, interp="linear")
    S = plan.num_slow_times
    x = reflectivity(scene.grid_shape[2], 500, 8.0, seed=7)
    phi_err = torch.from_numpy(np.cumsum(np.random.default_rng(8).standard_normal(S) * 0.3).astype(np.float32)).cuda()
    plan.set_slow_time_weighting(phase_weights(plan, phi_err))
    y = plan.forward(x)
    phi = torch.zeros(S, device="cuda")
    _, t = _suite_time(lambda: sharpness_gradient(plan, y, phi))
    return {"workload": "autofocus", "gradient_ms": t, "pixels": plan.num_scatterers, "pulses": S,
            "samples": plan.num_freqs}


def resample_workload() -> dict:
    import torch

    from sarsolver_gb300.geometry import NumpySimpleSarAperture, NumpySimpleSarDataset
    from sarsolver_gb300.resample import resample_dataset

    S = N = 8192
    az = np.deg2rad(np.linspace(-3, 3, S))
    tx = np.stack([10e3 * np.cos(az), 10e3 * np.sin(az), np.full(S, 5e3)], axis=-1)
    ap = NumpySimpleSarAperture(tx, tx, np.zeros((S, 3)), 10e9, 200e6, num_freqs=N)
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    ph = torch.complex(torch.randn(S, N, device="cuda", generator=g), torch.randn(S, N, device="cuda", generator=g))
    ds = NumpySimpleSarDataset(ap, ph)
    out, t = _suite_time(lambda: resample_dataset(ds, 2.0, 2, new_srp=np.array([5.0, 5.0, 0.0]), keep_on_device=True))
    return {"workload": "resample", "ms": t, "in": [S, N], "out": list(out.phase_history().shape)}


def pdhg_workload() -> dict:
    """100 PDHG iterations (f = ||A x - b||^2, g = 0; sigma = 1, tau = 1 / ||A||^2) on a held-out
    scene of the 512^2 x 1024 x 1024 learned-solver workload, against one forward projection plus
    one backprojection (the operator work of one iteration)."""
    import torch

    from sarsolver_gb300.learned import LearnedConfig, SceneSource
    from sarsolver_gb300.solvers import pdhg

    src = SceneSource(LearnedConfig(), seed=4242, continuous=True)
    plan, y, _, extent, snr = src.sample()
    _, norm_info = pdhg(plan, y, iterations=0, norm_iterations=50, tau=1.0)
    nrm = norm_info.operator_norm
    iters = 100
    (x, info), t = _suite_time(lambda: pdhg(plan, y, iterations=iters, sigma=1.0, tau=1.0 / nrm ** 2))
    xb = plan.adjoint(y)
    _, t_pair = _suite_time(lambda: plan.adjoint(plan.forward(xb)))
    return {"workload": "pdhg", "iterations": iters, "ms": t, "ms_per_iteration": t / iters,
            "operator_pair_ms": t_pair, "overhead_fraction": (t / iters - t_pair) / t_pair,
            "operator_norm": nrm, "residual_first": info.history[0], "residual_last": info.history[-1]}


def cphd_workload() -> dict:
    """8192 pulses x 8192 samples, CI4 with AmpSF (268 MB on disk): file -> complex64 on the device
    (warm page cache, wall clock), the decode kernel alone (CUDA events, HBM bytes), and the host
    decode of the same bytes with numpy big-endian types (what a host reader does)."""
    import torch

    import ctypes
    import os
    import tempfile
    import time

    from sarsolver_gb300 import _lib
    from sarsolver_gb300.cphd import FORMATS, Cphd101Dataset, write_cphd

    S = N = 8192
    rng = np.random.default_rng(11)
    az = np.deg2rad(np.linspace(-3, 3, S))
    tx = np.stack([10e3 * np.cos(az), 10e3 * np.sin(az), np.full(S, 5e3)], axis=-1)
    ph = (rng.standard_normal((S, N), dtype=np.float32) + 1j * rng.standard_normal((S, N), dtype=np.float32))
    out = {"workload": "cphd", "vectors": S, "samples": N, "format": "CI4"}
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "collection.cphd")
        write_cphd(path, [dict(phase_history=ph, trans_posns=tx, rec_posns=tx, srps=np.zeros((S, 3)),
                               centre_freq=10e9, sample_bandwidth=200e6)], signal_format="CI4", amp_sf=True)
        del ph
        out["file_bytes"] = os.path.getsize(path)
        ds = Cphd101Dataset(path)
        dst = torch.empty((S, N), dtype=torch.complex64, device="cuda")
        ds.phase_history_device(out=dst)   # warm the page cache and the allocator
        best = float("inf")
        for _ in range(3):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ds.phase_history_device(out=dst)
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t0)
        raw_bytes = S * N * FORMATS["CI4"][1]
        out["file_to_device_ms"] = best * 1e3
        out["file_to_device_gbs"] = raw_bytes / best / 1e9
        # decode kernel alone, raw bytes resident
        raw = torch.from_numpy(ds.reader.read_raw(slice(None)).reshape(-1)).cuda()
        amp = torch.from_numpy(ds.reader.amp_sf(0).astype(np.float32)).cuda()
        lib = _lib.load()
        st = torch.cuda.current_stream()

        def launch():
            _lib.check(lib.sar_cphd_decode(ctypes.c_void_p(raw.data_ptr()), _lib.SAR_CPHD_CI4, S, N,
                                           ctypes.c_void_p(amp.data_ptr()), ctypes.c_void_p(dst.data_ptr()),
                                           ctypes.c_void_p(st.cuda_stream)), "sar_cphd_decode")

        for _ in range(3):
            launch()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = 20
        e0.record(st)
        for _ in range(reps):
            launch()
        e1.record(st)
        torch.cuda.synchronize()
        k_ms = e0.elapsed_time(e1) / reps
        moved = raw_bytes + S * N * 8 + S * 4
        out["decode_kernel_ms"] = k_ms
        out["decode_kernel_gbs"] = moved / (k_ms * 1e-3) / 1e9
        # host decode of the same bytes (numpy big-endian int16 -> complex64, times AmpSF)
        host = ds.reader.read_raw(slice(None))
        a = ds.reader.amp_sf(0).astype(np.float32)
        t0 = time.perf_counter()
        comp = np.frombuffer(host.tobytes(), dtype=">i2").astype(np.float32).reshape(S, N, 2) * a[:, None, None]
        hc = np.empty((S, N), np.complex64)
        hc.real, hc.imag = comp[..., 0], comp[..., 1]
        out["host_decode_ms"] = (time.perf_counter() - t0) * 1e3
        out["decoded_equal"] = bool(np.array_equal(dst.cpu().numpy().view(np.uint32), hc.view(np.uint32)))
    return out


SETTINGS_ROWS = (("config2", "linear", 8.0, "auto"), ("config2_turned", "linear", 8.0, "auto"),
                 ("config2_diagonal", "linear", 8.0, "auto"), ("config2_steep", "linear", 8.0, "auto"),
                 ("config2", "nearest_ref", 8.0, "auto"),
                 ("config2", "linear", 128.0, "auto"), ("config2", "nearest_ref", 128.0, "auto"),
                 ("config2", "nearest_ref", 128.0, "points"))


def settings_workload(rows=SETTINGS_ROWS, verbose: bool = True) -> list:
    """The benchmark scene under other operator settings: linear / nearest_ref interpolation, upsample
    8 / 128 (the reference's default), and the collection turned by 90 degrees (range along y),
    looking along the grid diagonal or at 63.4 degrees to x.  Mean of 3 calls after one warm-up, CUDA events around each
    operator call."""
    import torch

    from sarsolver_gb300.plan import SarPlan
    from sarsolver_gb300.scenes import config_workload
    out = []
    for case, interp, U, path in rows:
        aperture, scene, _, _ = config_workload(case)
        plan = SarPlan(scene, aperture, upsample_ratio=U, interp=interp, path=path)
        g = torch.Generator(device="cuda")
        g.manual_seed(1)
        y = torch.complex(torch.randn(plan.num_slow_times, plan.num_freqs, device="cuda", generator=g),
                          torch.randn(plan.num_slow_times, plan.num_freqs, device="cuda", generator=g))
        x = torch.complex(torch.randn(plan.num_scatterers, device="cuda", generator=g),
                          torch.randn(plan.num_scatterers, device="cuda", generator=g))
        row = {"workload": "settings", "case": case, "interp": interp, "upsample": U, "path": path,
               "grid_path": plan.is_grid,
               "tile_window": plan.tile_window, "strip_window": plan.strip_window,
               "gather_lanes_y": plan.gather_lanes_y, "scatter_lanes_y": plan.scatter_lanes_y,
               "gather_shear": plan.gather_shear, "scatter_shear": plan.scatter_shear,
               "scatter_ring_half": plan.scatter_ring_half}
        for name, fn in (("adjoint_ms", lambda: plan.adjoint(y)), ("forward_ms", lambda: plan.forward(x))):
            fn()
            plan.enable_stage_timing(True)
            times = [_suite_time(fn, warmup=0)[1] for _ in range(3)]
            stages, calls = plan.stage_times()
            plan.enable_stage_timing(False)
            row[name] = sum(times) / len(times)
            # [FFT side before, main kernel, FFT side after] per call
            row[name.replace("_ms", "_stages_ms")] = [round(v / max(calls, 1), 3) for v in stages]
        assert plan.device_flags() == 0
        plan.close()
        del y, x
        torch.cuda.empty_cache()
        if verbose:
            print(json.dumps(row), flush=True)
        out.append(row)
    return out


def unet_workload(size: int = 512, batch: int = 1, iters: int = 10, warmup: int = 3, base_channels: int = 32) -> dict:
    """Forward and backward passes of the warm-start U-Net on a random complex image (CUDA events)."""
    import torch
    from sarsolver_gb300.unet import UNet

    net = UNet(base_channels, seed=0)
    g = torch.Generator(device="cuda")
    g.manual_seed(0)
    shape = (batch, size, size)
    x = torch.complex(torch.randn(shape, device="cuda", generator=g), torch.randn(shape, device="cuda", generator=g))
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    fwd = bwd = 0.0
    for i in range(warmup + iters):
        ev[0].record()
        y = net.forward(x)
        ev[1].record()
        net.zero_grad()
        net.backward(y)
        ev[2].record()
        torch.cuda.synchronize()
        if i >= warmup:
            fwd += ev[0].elapsed_time(ev[1])
            bwd += ev[1].elapsed_time(ev[2])
    # multiply-adds per pixel of the 15 convolutions at their levels (3x3 taps; 1x1 output layer)
    macs = 0.0
    for l in net.layers:
        macs += l["taps"] * (l["cin0"] + l["cin1"]) * l["cout"] / 4 ** l["level"]
    flops_fwd = 2.0 * macs * batch * size ** 2
    return {"workload": "unet", "size": size, "batch": batch, "base_channels": base_channels,
            "forward_ms": fwd / iters, "backward_ms": bwd / iters,
            "forward_tflops": flops_fwd / (fwd / iters * 1e-3) / 1e12,
            "backward_tflops": 2 * flops_fwd / (bwd / iters * 1e-3) / 1e12, "flags": net.flags()}


def run_suite(name: str) -> None:
    import torch

    torch.cuda.set_device(0)
    fn = {"cgls": cgls_workload, "autofocus": autofocus_workload, "resample": resample_workload,
          "cphd": cphd_workload, "pdhg": pdhg_workload, "settings": settings_workload, "unet": unet_workload}[name]
    res = fn()
    if not isinstance(res, list):   # the settings workload prints one line per setting itself
        print(json.dumps(res))


def main():
    args = parse()
    if args.suite:
        run_suite(args.suite)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
