"""CPU oracle of the learned initial guess's network (TEST INFRASTRUCTURE).

Only the tests, the smoke check and the benchmark's CPU leg import this
module; the product path runs the CUDA kernels of include/vdvc_cnn.h.

The reference has no learned seed (its multiscale solve seeds from coarse
levels and an FFT shift, engine/correlate_gpu.py:1143-1305), so there is no
reference behaviour to pin here.  This oracle restates the mathematics the
kernels implement -- 3x3x3 convolutions with zero padding, their adjoints and
weight gradients, linear 2x upsampling, the [1 2 2 2 1]/8 input low-pass,
mean squared error -- in float64 NumPy, and is itself pinned by
finite-difference checks (tests/test_cnn_oracle.py).  The convolution's
input gradient is written as a scatter (the literal adjoint of the forward
gather), independent of the gather form the CUDA kernels use.

Activations are (z, y, x, C) arrays; weights are (n_out, 27, cin) with tap
t = (tz*3 + ty)*3 + tx.  With bf16=True every value is rounded to BF16 where
the CUDA path stores BF16 (weights, input, stored activations and
activation gradients), so GPU and oracle differ only by FP32 accumulation.
"""
from __future__ import annotations

import numpy as np


def bf16_round(x):
    """Nearest BF16 value (ties to even) of float32(x), as float64."""
    b = np.ascontiguousarray(np.asarray(x, dtype=np.float32)).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def _r(x, bf16):
    return bf16_round(x) if bf16 else np.asarray(x, dtype=np.float64)


def tap_index(n_out, S, stride, t):
    """Source index of each output index for tap t of a stride-`stride`
    padding-1 convolution (-1 outside [0, S))."""
    q = np.arange(n_out) * stride - 1 + t
    return np.where((q >= 0) & (q < S), q, -1)


def conv(x, W, b, stride, relu):
    """y[p][n] = act(sum_{t,k} x[q(p,t)][k] W[n][t][k] + b[n]); x (Sz,Sy,Sx,C)."""
    Sz, Sy, Sx, C = x.shape
    n_out = W.shape[0]
    nz, ny, nx = ((Sz - 1) // stride + 1, (Sy - 1) // stride + 1, (Sx - 1) // stride + 1)
    y = np.zeros((nz, ny, nx, n_out))
    xp = np.zeros((Sz + 1, Sy + 1, Sx + 1, C))   # index -1 picks the zero plane
    xp[:Sz, :Sy, :Sx] = x
    for t in range(27):
        tx, ty, tz = t % 3, (t // 3) % 3, t // 9
        qz, qy, qx = tap_index(nz, Sz, stride, tz), tap_index(ny, Sy, stride, ty), tap_index(nx, Sx, stride, tx)
        xs = xp[np.ix_(qz, qy, qx)]          # -1 picks the zero plane
        y += xs @ W[:, t, :].T
    if b is not None:
        y += b
    return np.maximum(y, 0.0) if relu else y


def conv_input_grad(dy, W, stride, src_shape):
    """Adjoint of conv (before the activation): dx = sum over (p, t) of
    dy[p] W[:, t, :] scattered to x[q(p, t)]."""
    Sz, Sy, Sx = src_shape
    C = W.shape[2]
    nz, ny, nx = dy.shape[:3]
    dx = np.zeros((Sz + 1, Sy + 1, Sx + 1, C))
    for t in range(27):
        tx, ty, tz = t % 3, (t // 3) % 3, t // 9
        qz, qy, qx = tap_index(nz, Sz, stride, tz), tap_index(ny, Sy, stride, ty), tap_index(nx, Sx, stride, tx)
        contrib = dy @ W[:, t, :]
        np.add.at(dx, np.ix_(qz, qy, qx), contrib)
    return dx[:Sz, :Sy, :Sx]


def conv_wgrad(dy, x, stride):
    """dW[n][t][k] = sum_p dy[p][n] x[q(p,t)][k]; db[n] = sum_p dy[p][n]."""
    Sz, Sy, Sx, C = x.shape
    nz, ny, nx, n_out = dy.shape
    xp = np.zeros((Sz + 1, Sy + 1, Sx + 1, C))
    xp[:Sz, :Sy, :Sx] = x
    dW = np.zeros((n_out, 27, C))
    d2 = dy.reshape(-1, n_out)
    for t in range(27):
        tx, ty, tz = t % 3, (t // 3) % 3, t // 9
        qz, qy, qx = tap_index(nz, Sz, stride, tz), tap_index(ny, Sy, stride, ty), tap_index(nx, Sx, stride, tx)
        xs = xp[np.ix_(qz, qy, qx)].reshape(-1, C)
        dW[:, t, :] = d2.T @ xs
    return dW, d2.sum(axis=0)


def up_matrix(n, m):
    """(n, m) linear 2x upsampling along one axis (fine p reads coarse p/2,
    or the mean of (p-1)/2 and min((p+1)/2, m-1))."""
    U = np.zeros((n, m))
    for p in range(n):
        if p % 2 == 0:
            U[p, p // 2] += 1.0
        else:
            U[p, (p - 1) // 2] += 0.5
            U[p, min((p + 1) // 2, m - 1)] += 0.5
    return U


def upsample2(c, n_shape):
    Uz, Uy, Ux = (up_matrix(n, m) for n, m in zip(n_shape, c.shape[:3]))
    return np.einsum('zc,yb,xa,cbak->zyxk', Uz, Uy, Ux, c)


def upsample2_adjoint(df, m_shape):
    Uz, Uy, Ux = (up_matrix(n, m) for n, m in zip(df.shape[:3], m_shape))
    return np.einsum('zc,yb,xa,zyxk->cbak', Uz, Uy, Ux, df)


def pool_input(f, g, mean_std):
    """f, g: (nz, ny, nx) float arrays -> (gz, gy, gx, 2): the separable
    [1 2 2 2 1]/8 low-pass (renormalised at the borders) sampled every 4
    voxels, standardised by mean_std = (mean_f, std_f, mean_g, std_g)."""
    w = np.array([1.0, 2.0, 2.0, 2.0, 1.0])

    def axis_matrix(n):
        G = (n - 1) // 4 + 1
        A = np.zeros((G, n))
        for i in range(G):
            for d in range(-2, 3):
                v = 4 * i + d
                if 0 <= v < n:
                    A[i, v] = w[d + 2]
        return A

    Az, Ay, Ax = (axis_matrix(n) for n in f.shape)
    ones = np.ones_like(f, dtype=np.float64)
    norm = np.einsum('iz,jy,kx,zyx->ijk', Az, Ay, Ax, ones)
    pf = np.einsum('iz,jy,kx,zyx->ijk', Az, Ay, Ax, f.astype(np.float64)) / norm
    pg = np.einsum('iz,jy,kx,zyx->ijk', Az, Ay, Ax, g.astype(np.float64)) / norm
    mf, sf, mg, sg = mean_std
    return np.stack([(pf - mf) / sf, (pg - mg) / sg], axis=-1)


# ---- the network ---------------------------------------------------------------
#
# The 4-level encoder-decoder of voxeldvc_gb300/learned/arch.py:
#   e1 -> e2a -> e2b -> e3a -> e3b -> e4a -> e4b
#   d3 = conv([up(e4b) | e3b]),  d2 = conv([up(d3) | e2b]),  out = conv(d2)

def forward(params, x, layers, bf16=False):
    """params: {name: (W, b)}; x: (Gz, Gy, Gx, 2).  Returns (pred, cache)."""
    P = {k: (_r(W, bf16), np.asarray(b, dtype=np.float64)) for k, (W, b) in params.items()}
    L = {l["name"]: l for l in layers}

    def run(name, inp):
        l = L[name]
        return _r(conv(inp, P[name][0], P[name][1], l["stride"], l["relu"]), bf16)

    c = dict(P=P, x=_r(x, bf16))
    c["e1"] = run("e1", c["x"])
    c["e2a"] = run("e2a", c["e1"])
    c["e2b"] = run("e2b", c["e2a"])
    c["e3a"] = run("e3a", c["e2b"])
    c["e3b"] = run("e3b", c["e3a"])
    c["e4a"] = run("e4a", c["e3b"])
    c["e4b"] = run("e4b", c["e4a"])
    c["cat3"] = np.concatenate([_r(upsample2(c["e4b"], c["e3b"].shape[:3]), bf16), c["e3b"]], axis=-1)
    c["d3"] = run("d3", c["cat3"])
    c["cat2"] = np.concatenate([_r(upsample2(c["d3"], c["e2b"].shape[:3]), bf16), c["e2b"]], axis=-1)
    c["d2"] = run("d2", c["cat2"])
    l = L["out"]
    c["pred"] = conv(c["d2"], P["out"][0], P["out"][1], l["stride"], l["relu"])  # FP32 output on the GPU
    return c["pred"], c


def mse(pred, target):
    d = pred - target
    return float(np.mean(d * d)), 2.0 * d / d.size


def backward(cache, dpred, layers, bf16=False):
    """Gradients {name: (dW, db)} of the loss whose pred-gradient is dpred.
    Where two gradients meet (a skip connection), the GPU stores the first
    in BF16 and adds the second to it; the sum is rounded once more."""
    P = cache["P"]
    L = {l["name"]: l for l in layers}
    grads = {}

    def relu_mask(d, a):
        return np.where(a > 0, d, 0.0)

    def back(name, dy, x_in, want_dx=True):
        l = L[name]
        grads[name] = conv_wgrad(dy, x_in, l["stride"])
        if want_dx:
            return conv_input_grad(dy, P[name][0], l["stride"], x_in.shape[:3])
        return None

    c = cache
    dp = _r(dpred, bf16)
    dd2 = relu_mask(_r(back("out", dp, c["d2"]), bf16), c["d2"])
    dcat2 = _r(back("d2", dd2, c["cat2"]), bf16)
    c3 = c["d3"].shape[-1]
    dd3 = relu_mask(_r(upsample2_adjoint(dcat2[..., :c3], c["d3"].shape[:3]), bf16), c["d3"])
    dcat3 = _r(back("d3", dd3, c["cat3"]), bf16)
    c4 = c["e4b"].shape[-1]
    de4b = relu_mask(_r(upsample2_adjoint(dcat3[..., :c4], c["e4b"].shape[:3]), bf16), c["e4b"])
    de4a = relu_mask(_r(back("e4b", de4b, c["e4a"]), bf16), c["e4a"])
    de3b = relu_mask(_r(back("e4a", de4a, c["e3b"]) + dcat3[..., c4:], bf16), c["e3b"])
    de3a = relu_mask(_r(back("e3b", de3b, c["e3a"]), bf16), c["e3a"])
    de2b = relu_mask(_r(back("e3a", de3a, c["e2b"]) + dcat2[..., c3:], bf16), c["e2b"])
    de2a = relu_mask(_r(back("e2b", de2b, c["e2a"]), bf16), c["e2a"])
    de1 = relu_mask(_r(back("e2a", de2a, c["e1"]), bf16), c["e1"])
    back("e1", de1, c["x"], want_dx=False)
    return grads


def init_params(layers, seed=0):
    """He-normal weights (the last layer scaled by 0.1), zero biases."""
    rng = np.random.default_rng(seed)
    out = {}
    for i, l in enumerate(layers):
        std = np.sqrt(2.0 / (27 * l["cin"])) * (0.1 if i == len(layers) - 1 else 1.0)
        out[l["name"]] = (rng.standard_normal((l["cout"], 27, l["cin"])) * std, np.zeros(l["cout"]))
    return out
