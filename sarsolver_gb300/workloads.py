"""Run one of the library's workloads once and print its timing (for profiling and quick checks).

    python -m sarsolver_gb300.workloads cgls       # plain and learned CGLS, 512^2 x 1024 x 1024
    python -m sarsolver_gb300.workloads autofocus  # sharpness + phase gradient, 1024^2 x 2048 x 2048
    python -m sarsolver_gb300.workloads resample   # 8192 x 8192 phase history, factors 2 x 2

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


def main(argv=None) -> None:
    argv = sys.argv[1:] if argv is None else argv
    name = argv[0] if argv else "cgls"
    torch.cuda.set_device(0)
    fn = {"cgls": cgls_workload, "autofocus": autofocus_workload, "resample": resample_workload}[name]
    print(json.dumps(fn()))


if __name__ == "__main__":
    main()
