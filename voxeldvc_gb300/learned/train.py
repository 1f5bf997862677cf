"""Training of the learned initial guess, entirely on the GPU.

Pairs are made by the package's own generator (include/vdvc_synth.h): a
seeded 513^3 texture of the benchmark family (blurred white noise plus 5000
bright cylinders; a new texture every TEXTURE_EVERY pairs), a random
displacement field and the warped, noisy deformed image
g(x) = f(x - u(x)) + N(0, 0.01^2).  The field is
  * affine about the volume centre: a rotation of up to 5 degrees about a
    uniformly random axis, a symmetric strain with entries up to 3 % (the
    off-diagonal ones up to 1.5 %), a translation of up to 15 vx in a
    uniformly random direction;
  * plus a cubic B-spline displacement on a 16^3 control grid spanning the
    volume, control displacements uniform in [-A, A]^3 with the amplitude A
    itself uniform in [0, 4] vx per pair.
The target is the displacement a correlation recovers, U = u(X + U), on the
network's stride-8 output grid (the node grid of h = 8).  No necking field
is used, so the benchmark's field family is never seen in training.

Seeds: training pair k uses seed TRAIN_SEED_BASE + k, held-out pairs seeds
below HELD_OUT_LIMIT; the two ranges are disjoint.

    python -m voxeldvc_gb300.learned.train --pairs 20000 --batch 4 --out W.npz
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import time

import numpy as np

from .. import _device as D
from .. import _lib
from .. import synth
from .arch import grids, input_grid, OUT_STRIDE
from .seednet import SeedNet, WEIGHTS_PATH

TRAIN_SEED_BASE = 1_000_000
HELD_OUT_LIMIT = 100_000
SIZE = 513
N_CYL = 5000
TEXTURE_EVERY = 4
CONTROL = 16
MAX_ROT_DEG, MAX_STRAIN, MAX_SHIFT, MAX_SPLINE = 5.0, 0.03, 15.0, 4.0


def random_field(rng, size=SIZE):
    """(affine t[3] + G[9] + c[3] float64, control displacements (nc^3, 3)
    float32) of one pair."""
    axis = rng.standard_normal(3)
    axis /= np.linalg.norm(axis)
    th = np.deg2rad(rng.uniform(0.0, MAX_ROT_DEG))
    Kx = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    R = np.eye(3) + np.sin(th) * Kx + (1 - np.cos(th)) * Kx @ Kx
    E = np.diag(rng.uniform(-MAX_STRAIN, MAX_STRAIN, 3))
    off = rng.uniform(-MAX_STRAIN / 2, MAX_STRAIN / 2, 3)
    E[0, 1] = E[1, 0] = off[0]
    E[0, 2] = E[2, 0] = off[1]
    E[1, 2] = E[2, 1] = off[2]
    G = R @ (np.eye(3) + E) - np.eye(3)
    d = rng.standard_normal(3)
    t = d / np.linalg.norm(d) * rng.uniform(0.0, MAX_SHIFT)
    c = (size - 1) / 2.0
    affine = np.concatenate([t, G.reshape(-1), [c, c, c]])
    amp = rng.uniform(0.0, MAX_SPLINE)
    ctrl = rng.uniform(-amp, amp, (CONTROL ** 3, 3)).astype(np.float32)
    return affine, ctrl


class PairMaker:
    """Generates training / held-out pairs on the GPU, reusing one texture
    for consecutive pairs that name the same texture seed."""

    def __init__(self, size=SIZE, n_cyl=N_CYL, noise=0.01):
        self.size, self.n_cyl, self.noise = size, n_cyl, noise
        self.shape = (size, size, size)
        self._tex_key = None
        self._f = None
        self.g = D.empty(size ** 3, np.float32)
        self.n = grids(input_grid(self.shape))[1]
        self.target = D.empty(int(np.prod(self.n)) * 3, np.float32)

    def make(self, seed, texture_seed=None):
        """(f_vox, g_vox, shape, target (npos(G1) * 3) float32 CUDA)."""
        texture_seed = seed if texture_seed is None else texture_seed
        if texture_seed != self._tex_key:
            self._f = synth.texture(self.shape, self.n_cyl, seed=texture_seed, cyl_seed=texture_seed + 7)
            self._tex_key = texture_seed
        rng = np.random.default_rng(seed)
        affine, ctrl = random_field(rng, self.size)
        L = _lib.lib()
        aff = np.ascontiguousarray(affine, np.float64)
        ctrl_d = D.to_device(ctrl.reshape(-1))
        s = self.size
        _lib.check(L.vdvc_synth_warp_ffd(self._f.data_ptr(), s, s, s, aff.ctypes.data_as(_lib.pd), ctrl_d.data_ptr(),
                                         CONTROL, self.noise, C.c_ulonglong(seed + 13), self.g.data_ptr(),
                                         D.stream()), "synth_warp_ffd")
        _lib.check(L.vdvc_synth_ffd_inverse_grid(aff.ctypes.data_as(_lib.pd), ctrl_d.data_ptr(), CONTROL, s, s, s,
                                                 *self.n, float(OUT_STRIDE), 30, self.target.data_ptr(), D.stream()),
                   "synth_ffd_inverse_grid")
        D.torch().cuda.current_stream().synchronize()  # ctrl_d is freed on return
        return self._f, self.g, self.shape, self.target


def validate(net, maker, n_pairs=16):
    """RMS error (vx) of the prediction on held-out pairs, and the RMS of
    the fields themselves (the error of a zero seed)."""
    err, mag = [], []
    for i in range(n_pairs):
        f, g, shape, target = maker.make(HELD_OUT_LIMIT - 1 - i)
        G = net.set_input(f, g, shape)
        net.forward(G)
        err.append(math.sqrt(float(net.loss(G, target, want_grad=False).item())))
        mag.append(float(np.sqrt(np.mean(target.cpu().numpy().astype(np.float64) ** 2))))
    return float(np.mean(err)), float(np.mean(mag))


def train(pairs=20000, batch=4, lr=3e-4, seed=0, log_every=100, out=WEIGHTS_PATH, log=print, clip=1.0):
    """Adam over `pairs` on-the-fly pairs in batches of `batch`: linear
    warm-up over the first thirtieth of the steps, then a cosine decay; the
    batch gradient is clipped to an L2 norm of `clip` (fields of up to ~40
    vx make single batches' gradients vary by orders of magnitude, and
    without the clip the network settles on predicting zero)."""
    torch = D.torch()
    net = SeedNet(seed=seed)
    maker = PairMaker()
    steps = max(1, pairs // batch)
    warm = max(1, steps // 30)
    t0 = time.perf_counter()
    history = []
    for step in range(1, steps + 1):
        lr_t = lr * min(1.0, step / warm) * 0.5 * (1.0 + math.cos(math.pi * step / steps))
        for bi in range(batch):
            k = (step - 1) * batch + bi
            f, g, shape, target = maker.make(TRAIN_SEED_BASE + k, texture_seed=TRAIN_SEED_BASE + k // TEXTURE_EVERY)
            G = net.set_input(f, g, shape)
            net.forward(G)
            loss = net.loss(G, target, scale=1.0 / batch)
            net.backward(G, accumulate=bi > 0)
        if clip:
            gn = torch.linalg.vector_norm(net.grad)
            net.grad.mul_(torch.clamp(clip / (gn + 1e-12), max=1.0))
        net.adam(max(lr_t, lr * 1e-3))
        if step % log_every == 0 or step == steps:
            _lib.check(_lib.lib().vdvc_cnn_status(D.stream()), "tensor-core convolutions")
            l = float(loss.item())
            history.append((step, l))
            log(f"step {step:5d}  loss {l:.4f} vx^2  ({time.perf_counter() - t0:.0f} s)", flush=True)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    val_rms, val_mag = validate(net, maker)
    log(f"held-out RMS error {val_rms:.3f} vx (field RMS {val_mag:.3f} vx); training {train_s:.0f} s")
    if out:
        net.save(out, pairs=steps * batch, batch=batch, lr=lr, clip=clip, size=SIZE, seed=seed, train_seconds=train_s,
                 val_rms=val_rms, val_field_rms=val_mag, history=np.asarray(history, np.float64))
    return net, dict(val_rms=val_rms, val_field_rms=val_mag, train_seconds=train_s, pairs=steps * batch,
                     history=history)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--pairs", type=int, default=20000)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--lr", type=float, default=3e-4)
    ap.add_argument("--clip", type=float, default=1.0, help="L2 norm the batch gradient is clipped to (0: none)")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--log-every", type=int, default=100)
    ap.add_argument("--out", default=WEIGHTS_PATH)
    a = ap.parse_args(argv)
    _, info = train(a.pairs, a.batch, a.lr, a.seed, a.log_every, a.out, clip=a.clip)
    print(json.dumps({k: v for k, v in info.items() if k != "history"}))


if __name__ == "__main__":
    main()
