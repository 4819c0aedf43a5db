"""Trains the pressure warm-start U-Net on snapshots this solver generates.

    python -m stroemung_gb300.train_warmstart --snapshots 20000 --epochs 12 \\
        --out weights.npy --log train.json

Snapshots: seeded 512 x 128 channels (4..32 no-slip rectangles with sides of
4..32 cells placed by the channel workload's rules, Reynolds number
log-uniform in [50, 1000], u = 1 at t = 0) stepped by the mixed-precision
solver; every step contributes its RHS, flags and previous pressure (the
network's input) and the pressure its solve reached (the target).  Training:
Adam (lr 1e-3 by default), batch 32, on the library's tcgen05 forward /
backward kernels and its Adam kernel, with one of two losses (--loss):
`residual`, the relative Poisson residual of the corrected pressure
(sum r^2 / sum rhs^2), or `error`, its relative error against the solved
pressure (mean-free on fluid cells).  A held-out set from other seeds
measures both before and after training.

Writes the network's BF16 parameters (the values its forward uses; loading
them gives the same predictions) as a uint16 .npy, and a JSON log with the
loss of every epoch, the held-out measurements, timings and the SHA-256 of
the parameter file.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import time
from pathlib import Path

import numpy as np


def save_bf16(net, path: Path) -> str:
    """The network's BF16 parameters as uint16; returns their SHA-256."""
    bits = net.theta_bf.detach().view(dtype=__import__("torch").int16).cpu().numpy()
    arr = bits.view(np.uint16)
    np.save(path, arr)
    return hashlib.sha256(arr.tobytes()).hexdigest()


def bf16_bits_to_f32(bits: np.ndarray) -> np.ndarray:
    """BF16 values stored as uint16 bit patterns -> the same values as
    float32 (exact: BF16 is the top half of an FP32)."""
    return (np.asarray(bits, dtype=np.uint16).astype(np.uint32) << 16).view(np.float32)


def load_weights(net, path) -> str:
    """Loads parameters saved by save_bf16 (uint16 BF16 bits) or FP32
    parameters (float32); returns the SHA-256 of the stored array."""
    arr = np.load(path)
    theta = bf16_bits_to_f32(arr) if arr.dtype == np.uint16 else arr.astype(np.float32)
    net.load_state_dict({"theta": theta, "step": 1})
    return hashlib.sha256(arr.tobytes()).hexdigest()


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--snapshots", type=int, default=20000)
    ap.add_argument("--held-out", type=int, default=256)
    ap.add_argument("--steps-per-problem", type=int, default=25)
    ap.add_argument("--epochs", type=int, default=12)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=21)
    ap.add_argument("--loss", choices=["residual", "error"], default="residual")
    ap.add_argument("--out", required=True, help="parameter file (.npy)")
    ap.add_argument("--log", default="", help="JSON log (default: printed)")
    args = ap.parse_args(argv)

    import torch
    from . import warmstart
    from .unet import UNet

    t0 = time.perf_counter()
    train = warmstart.generate_snapshots(args.snapshots, imax=512, jmax=128,
                                         steps_per_problem=args.steps_per_problem,
                                         seed=args.seed, targets=True)
    held = warmstart.generate_snapshots(args.held_out, imax=512, jmax=128,
                                        steps_per_problem=args.steps_per_problem,
                                        seed=args.seed + 1000, targets=True)
    torch.cuda.synchronize()
    t_gen = time.perf_counter() - t0

    net = UNet(seed=args.seed)
    err = warmstart.Trainer(net, 514, 130, 0.01, 0.01, batch=args.batch, loss="error")
    res = warmstart.Trainer(net, 514, 130, 0.01, 0.01, batch=args.batch, loss="residual")

    def held_out():
        e, r = [], []
        for s0 in range(0, args.held_out - args.batch + 1, args.batch):
            e.append(err.loss(held, s0)[0])
            r.append(res.loss(held, s0)[0])
        return float(np.mean(e)), float(np.mean(r))

    before = held_out()
    trainer = err if args.loss == "error" else res
    epochs = []
    t0 = time.perf_counter()
    for ep in range(args.epochs):
        te = time.perf_counter()
        hist = trainer.fit(train, epochs=1, lr=args.lr, seed=args.seed + ep)
        torch.cuda.synchronize()
        he, hr = held_out()
        epochs.append({"epoch": ep, "train_loss": float(np.mean(hist)),
                       "held_out_error_loss": he, "held_out_relative_residual": hr,
                       "s": time.perf_counter() - te})
        print(json.dumps(epochs[-1]), flush=True)
    t_train = time.perf_counter() - t0
    out = Path(args.out)
    sha = save_bf16(net, out)
    log = {"snapshots": args.snapshots, "grid": "512x128", "held_out": args.held_out,
           "steps_per_problem": args.steps_per_problem, "batch": args.batch, "lr": args.lr,
           "epochs": args.epochs, "adam_steps": net.step, "params": net.parameter_count(),
           "loss": args.loss,
           "held_out_before": {"error_loss": before[0], "relative_residual": before[1]},
           "held_out_after": {"error_loss": epochs[-1]["held_out_error_loss"] if epochs
                              else before[0],
                              "relative_residual": epochs[-1]["held_out_relative_residual"]
                              if epochs else before[1]},
           "per_epoch": epochs, "generate_s": t_gen, "train_s": t_train,
           "train_ms_per_adam_step": t_train / max(net.step, 1) * 1e3,
           "weights": out.name, "weights_sha256": sha}
    text = json.dumps(log)
    if args.log:
        Path(args.log).write_text(text + "\n")
    print(text)


if __name__ == "__main__":
    main()
