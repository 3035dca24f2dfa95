"""Training data and training of the learned BBPGD warm start.

The network (see ``include/alens_gpu.h``, "Learned warm start") is trained
on (feature, converged multiplier) pairs that the FP64 solver itself
produces: seeded 3D systems shaped like the plain 1,000-rod periodic case
(lengths U[0.5, 1.0] um, diameter 0.025 um, isotropic, the same number
density) scaled up to 20,000 rods, stepped with the FP64 solver while the
library records every collision constraint's features before the solve and
its converged multiplier after it.  Training uses the library's own forward,
backward and Adam kernels.

Usage as a script::

    python -m alens_gb300.warmstart --samples 10000000 --out weights.npy
"""
from __future__ import annotations

import argparse
import math
import time

import numpy as np

from . import capi, workloads


def config1_shaped(n: int, seed: int, **kw) -> workloads.Workload:
    """Periodic cube with the number density of 1,000 rods in 5^3 um^3."""
    side = 5.0 * (n / 1000.0) ** (1.0 / 3.0)
    return workloads.small_periodic(n=n, box=side, seed=seed, **kw)


def generate(mlp: capi.Mlp, samples: int, rods: int = 20000, seeds=(101, 102, 103, 104),
             relax_steps: int = 5, max_steps: int = 100000, systems=None) -> dict:
    """Fill the model's dataset with up to `samples` rows from FP64 runs.

    The steps of each seeded system are taken in turn (round robin) so that
    early (overlapped) and later (relaxed) states are both represented.
    `systems` may give workloads to use instead of the config-1-shaped
    ones."""
    ws = systems if systems is not None else [config1_shaped(rods, s) for s in seeds]
    gs = []
    for w in ws:
        cfg = workloads.config_with(w.cfg, precision=capi.PREC_FP64, warmStart=capi.WARM_PREV)
        g = capi.GpuSystem(cfg)
        g.set_rods(w.rods)
        g.set_feature_capture(True)
        for _ in range(relax_steps):
            g.step()
        gs.append(g)
    t0 = time.perf_counter()
    steps = 0
    start = mlp.dataset_size()
    while mlp.dataset_size() - start < samples and steps < max_steps:
        g = gs[steps % len(gs)]
        g.step()
        g.collect(mlp)
        steps += 1
    for g in gs:
        g.close()
    return {"rows": mlp.dataset_size() - start, "steps": steps, "systems": len(ws),
            "seconds": time.perf_counter() - t0}


def train(mlp: capi.Mlp, epochs: int = 20, batch: int = 65536, lr: float = 1e-3, seed: int = 0) -> dict:
    t0 = time.perf_counter()
    loss = mlp.train(epochs, batch=batch, lr=lr, seed=seed)
    return {"epochs": epochs, "batch": batch, "lr": lr, "loss_first": float(loss[0]),
            "loss_last": float(loss[-1]), "seconds": time.perf_counter() - t0}


def build_model(samples: int = 2_000_000, epochs: int = 20, seed: int = 0, rods: int = 20000) -> tuple:
    """Generate data from FP64 runs and train a model; returns (model, info)."""
    mlp = capi.Mlp(seed=seed, capacity=samples)
    info = {"generate": generate(mlp, samples, rods=rods)}
    info["train"] = train(mlp, epochs=epochs, seed=seed)
    info["samples"] = mlp.dataset_size()
    return mlp, info


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--samples", type=int, default=10_000_000)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=None, help="save the trained FP32 parameters (.npy)")
    a = ap.parse_args()
    mlp, info = build_model(a.samples, a.epochs, a.seed)
    print(info)
    if a.out:
        np.save(a.out, mlp.params())


if __name__ == "__main__":
    main()
