"""Train the learned CGLS warm start on generated scenes and compare it with plain CGLS.

    python -m sarsolver_gb300.train_warmstart --scenes 20000 --out sarsolver_gb300/weights/unet_warmstart.pt

Training scenes come from one seeded source (aperture extents on a 0.25-degree grid of cached
plans), evaluation scenes from another seed with continuous extents.  The checkpoint holds the
network width, the flat FP32 parameter vector, the workload and the training log; the comparison
prints one JSON line per scene and a summary line.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import time

import numpy as np
import torch

from .learned import LearnedConfig, SceneSource, WarmStart, compare, train
from .unet import UNet

DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "unet_warmstart.pt")


def load_warm_start(path: str = DEFAULT_WEIGHTS, device=None):
    """(WarmStart, LearnedConfig) from a checkpoint written by this module."""
    state = torch.load(path, map_location="cpu", weights_only=False)
    cfg = LearnedConfig(**state["config"])
    net = UNet(base_channels=int(state["base_channels"]), device=device)
    net.set_params(state["params"])
    return WarmStart(net, cfg.n), cfg


def summary(records) -> dict:
    plain_ms = float(np.mean([r.plain_ms for r in records]))
    learned_ms = float(np.mean([r.learned_ms for r in records]))
    return {
        "scenes": len(records),
        "plain_ms": plain_ms,
        "learned_ms": learned_ms,
        "speedup": plain_ms / learned_ms,
        "plain_iterations": float(np.mean([r.plain_iterations for r in records])),
        "learned_iterations": float(np.mean([r.learned_iterations for r in records])),
        "warm_start_residual": float(np.mean([r.start_residual for r in records])),
        "all_converged": bool(all(r.plain_converged and r.learned_converged for r in records)),
        **({"truth_start_iterations": float(np.mean([r.truth_iterations for r in records])),
            "truth_start_ms": float(np.mean([r.truth_ms for r in records])),
            "truth_start_residual": float(np.mean([r.truth_start_residual for r in records])),
            "warm_start_ceiling_speedup": plain_ms / float(np.mean([r.truth_ms for r in records]))}
           if records and np.isfinite(records[0].truth_ms) else {}),
    }


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--scenes", type=int, default=20000)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--base-channels", type=int, default=32)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--eval", type=int, default=16, help="held-out scenes for the comparison")
    ap.add_argument("--out", default=DEFAULT_WEIGHTS)
    ap.add_argument("--init", default=None, help="start from this checkpoint")
    ap.add_argument("--tol", type=float, default=1e-3)
    ap.add_argument("--loss", choices=["normal", "data", "truth"], default="normal",
                    help="training loss (WarmStart.loss): normal-equations residual, data residual, or "
                         "data-domain error against the noise-free scene")
    args = ap.parse_args(argv)

    torch.cuda.set_device(0)
    cfg = LearnedConfig()
    net = UNet(base_channels=args.base_channels, seed=args.seed, zero_output=True)
    if args.init:
        state = torch.load(args.init, map_location="cpu", weights_only=False)
        net.set_params(state["params"])
    warm = WarmStart(net, cfg.n)
    src = SceneSource(cfg, seed=1000 + args.seed)
    log = train(net, src, args.scenes, batch=args.batch, lr=args.lr, warm=warm, loss=args.loss,
                printer=lambda s: print(s, flush=True)) if args.scenes > 0 else None
    src.close()
    if net.flags():
        raise RuntimeError("a U-Net kernel reported a wait timeout")
    if log is not None:
        os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
        # bf16 is what the kernels use for the filters; biases lose nothing that matters.
        torch.save({"base_channels": args.base_channels, "params": net.params().cpu().to(torch.bfloat16),
                    "config": dataclasses.asdict(cfg), "loss": args.loss,
                    "log": {"steps": log.steps, "loss": log.loss, "scenes": log.scenes, "seconds": log.seconds}},
                   args.out)
        print(json.dumps({"trained_scenes": log.scenes, "seconds": round(log.seconds, 1),
                          "final_loss": log.loss[-1] if log.loss else None, "out": args.out}), flush=True)
    if args.eval:
        test = SceneSource(cfg, seed=99991, continuous=True)
        compare(warm, test, 1, tol=args.tol)    # warm-up (plans, cuFFT, module loads)
        recs = compare(warm, test, args.eval, tol=args.tol, repeats=2, truth=True)
        for r in recs:
            print(json.dumps(dataclasses.asdict(r)), flush=True)
        print(json.dumps({"summary": summary(recs)}), flush=True)
        test.close()


if __name__ == "__main__":
    main()
