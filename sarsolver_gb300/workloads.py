"""Run one of the library's workloads once and print its timing (for profiling and quick checks).

    python -m sarsolver_gb300.workloads cgls       # plain and learned CGLS, 512^2 x 1024 x 1024
    python -m sarsolver_gb300.workloads autofocus  # sharpness + phase gradient, 1024^2 x 2048 x 2048
    python -m sarsolver_gb300.workloads resample   # 8192 x 8192 phase history, factors 2 x 2
    python -m sarsolver_gb300.workloads cphd       # 8192 x 8192 CI4 CPHD file -> device
    python -m sarsolver_gb300.workloads pdhg       # 100 PDHG iterations, 512^2 x 1024 x 1024
    python -m sarsolver_gb300.workloads settings   # one backprojection + one forward projection at
                                                   # 2048^2 x 4096 x 4096 per interpolation mode,
                                                   # upsample factor and collection direction

Each prints one JSON line with CUDA-event times of the timed call (after one warm-up call).
"""
from __future__ import annotations

import json
import sys

import numpy as np
import torch


def _time(fn, warmup: int = 1):
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
    from .learned import LearnedConfig, SceneSource
    from .solvers import cgls
    from .train_warmstart import DEFAULT_WEIGHTS, load_warm_start

    warm, cfg = load_warm_start(DEFAULT_WEIGHTS)
    src = SceneSource(cfg if isinstance(cfg, LearnedConfig) else LearnedConfig(), seed=31337, continuous=True)
    plan, y, _, extent, snr = src.sample()
    (_, plain), t_plain = _time(lambda: cgls(plan, y, tol=1e-3, max_iterations=500))
    (_, learned), t_learned = _time(lambda: warm.solve(plan, y, tol=1e-3, max_iterations=500))
    return {"workload": "cgls", "extent_deg": extent, "snr_db": snr, "plain_ms": t_plain,
            "plain_iterations": plain.iterations, "learned_ms": t_learned, "learned_iterations": learned.iterations}


def autofocus_workload() -> dict:
    from .autodiff import phase_weights, sharpness_gradient
    from .plan import SarPlan
    from .scenes import config_workload, reflectivity

    aperture, scene, upsample, _ = config_workload("config3")
    plan = SarPlan(scene, aperture, upsample_ratio=upsample, interp="linear")
    S = plan.num_slow_times
    x = reflectivity(scene.grid_shape[2], 500, 8.0, seed=7)
    phi_err = torch.from_numpy(np.cumsum(np.random.default_rng(8).standard_normal(S) * 0.3).astype(np.float32)).cuda()
    plan.set_slow_time_weighting(phase_weights(plan, phi_err))
    y = plan.forward(x)
    phi = torch.zeros(S, device="cuda")
    _, t = _time(lambda: sharpness_gradient(plan, y, phi))
    return {"workload": "autofocus", "gradient_ms": t, "pixels": plan.num_scatterers, "pulses": S,
            "samples": plan.num_freqs}


def resample_workload() -> dict:
    from .geometry import NumpySimpleSarAperture, NumpySimpleSarDataset
    from .resample import resample_dataset

    S = N = 8192
    az = np.deg2rad(np.linspace(-3, 3, S))
    tx = np.stack([10e3 * np.cos(az), 10e3 * np.sin(az), np.full(S, 5e3)], axis=-1)
    ap = NumpySimpleSarAperture(tx, tx, np.zeros((S, 3)), 10e9, 200e6, num_freqs=N)
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    ph = torch.complex(torch.randn(S, N, device="cuda", generator=g), torch.randn(S, N, device="cuda", generator=g))
    ds = NumpySimpleSarDataset(ap, ph)
    out, t = _time(lambda: resample_dataset(ds, 2.0, 2, new_srp=np.array([5.0, 5.0, 0.0]), keep_on_device=True))
    return {"workload": "resample", "ms": t, "in": [S, N], "out": list(out.phase_history().shape)}


def pdhg_workload() -> dict:
    """100 PDHG iterations (f = ||A x - b||^2, g = 0; sigma = 1, tau = 1 / ||A||^2) on a held-out
    scene of the 512^2 x 1024 x 1024 learned-solver workload, against one forward projection plus
    one backprojection (the operator work of one iteration)."""
    from .learned import LearnedConfig, SceneSource
    from .solvers import pdhg

    src = SceneSource(LearnedConfig(), seed=4242, continuous=True)
    plan, y, _, extent, snr = src.sample()
    _, norm_info = pdhg(plan, y, iterations=0, norm_iterations=50, tau=1.0)
    nrm = norm_info.operator_norm
    iters = 100
    (x, info), t = _time(lambda: pdhg(plan, y, iterations=iters, sigma=1.0, tau=1.0 / nrm ** 2))
    xb = plan.adjoint(y)
    _, t_pair = _time(lambda: plan.adjoint(plan.forward(xb)))
    return {"workload": "pdhg", "iterations": iters, "ms": t, "ms_per_iteration": t / iters,
            "operator_pair_ms": t_pair, "overhead_fraction": (t / iters - t_pair) / t_pair,
            "operator_norm": nrm, "residual_first": info.history[0], "residual_last": info.history[-1]}


def cphd_workload() -> dict:
    """8192 pulses x 8192 samples, CI4 with AmpSF (268 MB on disk): file -> complex64 on the device
    (warm page cache, wall clock), the decode kernel alone (CUDA events, HBM bytes), and the host
    decode of the same bytes with numpy big-endian types (what a host reader does)."""
    import ctypes
    import os
    import tempfile
    import time

    from . import _lib
    from .cphd import FORMATS, Cphd101Dataset, write_cphd

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


def settings_workload() -> list:
    """The benchmark scene under other operator settings: linear / nearest_ref interpolation, upsample
    8 / 128 (the reference's default), and the collection turned by 90 degrees (range along y).
    Mean of 3 calls after one warm-up, CUDA events around each operator call."""
    from .plan import SarPlan
    from .scenes import config_workload
    out = []
    for case, interp, U, path in (("config2", "linear", 8.0, "auto"), ("config2_turned", "linear", 8.0, "auto"),
                                  ("config2_diagonal", "linear", 8.0, "auto"),
                                  ("config2", "nearest_ref", 8.0, "auto"), ("config2", "linear", 128.0, "auto"),
                                  ("config2", "nearest_ref", 128.0, "auto"), ("config2", "nearest_ref", 128.0, "points")):
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
               "gather_lanes_y": plan.gather_lanes_y, "scatter_lanes_y": plan.scatter_lanes_y}
        for name, fn in (("adjoint_ms", lambda: plan.adjoint(y)), ("forward_ms", lambda: plan.forward(x))):
            fn()
            plan.enable_stage_timing(True)
            times = [_time(fn, warmup=0)[1] for _ in range(3)]
            stages, calls = plan.stage_times()
            plan.enable_stage_timing(False)
            row[name] = sum(times) / len(times)
            # [FFT side before, main kernel, FFT side after] per call
            row[name.replace("_ms", "_stages_ms")] = [round(v / max(calls, 1), 3) for v in stages]
        assert plan.device_flags() == 0
        plan.close()
        del y, x
        torch.cuda.empty_cache()
        print(json.dumps(row), flush=True)
        out.append(row)
    return out


def main(argv=None) -> None:
    argv = sys.argv[1:] if argv is None else argv
    name = argv[0] if argv else "cgls"
    torch.cuda.set_device(0)
    fn = {"cgls": cgls_workload, "autofocus": autofocus_workload, "resample": resample_workload,
          "cphd": cphd_workload, "pdhg": pdhg_workload, "settings": settings_workload}[name]
    res = fn()
    if not isinstance(res, list):   # the settings workload prints one line per setting itself
        print(json.dumps(res))


if __name__ == "__main__":
    main()
