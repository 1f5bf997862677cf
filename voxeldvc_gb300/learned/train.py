"""Training of the learned initial guess, entirely on the GPU.

Pairs are made by the package's own generator (include/vdvc_synth.h): a
seeded texture of the benchmark family (blurred white noise plus bright
cylinders, 257^3 voxels), a random smooth field -- translation up to
+-10 vx, a random displacement gradient (entries up to +-0.025) and up to
four Gaussian bumps of up to +-3 vx with widths 30-90 vx -- and the warped,
noisy deformed image g(x) = f(x - u(x)) + N(0, 0.01^2).  The target is the
field on the network's stride-8 output grid.  No necking field is used, so
the benchmark's field family is never seen in training.

Seeds: training pairs use seeds from TRAIN_SEED_BASE upward, the held-out
pairs of `validate` seeds below VAL_SEED_LIMIT; the two ranges are disjoint.

    python -m voxeldvc_gb300.learned.train --steps 3000 --batch 4 --out W.npz
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np

from .. import _device as D
from .. import synth
from .arch import grids, input_grid, OUT_STRIDE
from .seednet import SeedNet, WEIGHTS_PATH

TRAIN_SEED_BASE = 1_000_000
VAL_SEED_LIMIT = 100_000


def random_field(rng, size):
    """Parameters of a FIELD_BUMPS displacement for a size^3 volume."""
    c = (size - 1) / 2.0
    t = rng.uniform(-10.0, 10.0, 3)
    G = rng.uniform(-0.025, 0.025, (3, 3))
    nb = int(rng.integers(0, 5))
    params = [*t, *G.reshape(-1), c, c, c, float(nb)]
    for _ in range(nb):
        params += [*rng.uniform(0, size - 1, 3), float(rng.uniform(30.0, 90.0)), *rng.uniform(-3.0, 3.0, 3)]
    return params


def make_pair(seed, size=257, noise=0.01):
    """(f_vox, g_vox, shape, target (npos(n), 3) float32 CUDA, params)."""
    rng = np.random.default_rng(seed)
    shape = (size, size, size)
    n_cyl = int(round(5000 * (size / 513) ** 3))
    f = synth.texture(shape, n_cyl, seed=seed, cyl_seed=seed + 7)
    params = random_field(rng, size)
    g = synth.warp(f, shape, synth.FIELD_BUMPS, params, noise, seed=seed + 13)
    n = grids(input_grid(shape))[1]
    target = synth.field_grid(synth.FIELD_BUMPS, params, n, OUT_STRIDE)
    return f, g, shape, target, params


def validate(net, n_pairs=8, size=257):
    """RMS error (vx) of the prediction on held-out pairs, and the RMS of
    the fields themselves (the error of a zero seed)."""
    err, mag = [], []
    for i in range(n_pairs):
        f, g, shape, target, _ = make_pair(VAL_SEED_LIMIT - 1 - i, size)
        G = net.set_input(f, g, shape)
        net.forward(G)
        err.append(math.sqrt(float(net.loss(G, target, want_grad=False).item())))
        mag.append(float(np.sqrt(np.mean(target.cpu().numpy().astype(np.float64) ** 2))))
    return float(np.mean(err)), float(np.mean(mag))


def train(steps=3000, batch=4, lr=1e-3, size=257, seed=0, log_every=100, out=WEIGHTS_PATH, log=print):
    torch = D.torch()
    net = SeedNet(seed=seed)
    warm = max(1, steps // 30)
    t0 = time.perf_counter()
    history = []
    for step in range(1, steps + 1):
        lr_t = lr * min(1.0, step / warm) * 0.5 * (1.0 + math.cos(math.pi * step / steps))
        for bi in range(batch):
            f, g, shape, target, _ = make_pair(TRAIN_SEED_BASE + (step - 1) * batch + bi, size)
            G = net.set_input(f, g, shape)
            net.forward(G)
            loss = net.loss(G, target, scale=1.0 / batch)
            net.backward(G, accumulate=bi > 0)
        net.adam(max(lr_t, lr * 1e-3))
        if step % log_every == 0 or step == steps:
            l = float(loss.item())
            history.append((step, l))
            log(f"step {step:5d}  loss {l:.4f} vx^2  ({time.perf_counter() - t0:.0f} s)")
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    val_rms, val_mag = validate(net, size=size)
    log(f"held-out RMS error {val_rms:.3f} vx (field RMS {val_mag:.3f} vx); training {train_s:.0f} s")
    if out:
        net.save(out, steps=steps, batch=batch, lr=lr, size=size, seed=seed, train_seconds=train_s,
                 val_rms=val_rms, val_field_rms=val_mag, history=np.asarray(history, np.float64))
    return net, dict(val_rms=val_rms, val_field_rms=val_mag, train_seconds=train_s, history=history)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--size", type=int, default=257)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--log-every", type=int, default=100)
    ap.add_argument("--out", default=WEIGHTS_PATH)
    a = ap.parse_args(argv)
    _, info = train(a.steps, a.batch, a.lr, a.size, a.seed, a.log_every, a.out)
    print(json.dumps({k: v for k, v in info.items() if k != "history"}))


if __name__ == "__main__":
    main()
