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

def forward(params, x, layers, bf16=False):
    """params: {name: (W, b)}; x: (Gz, Gy, Gx, 2).  Returns (pred, cache)."""
    P = {k: (_r(W, bf16), np.asarray(b, dtype=np.float64)) for k, (W, b) in params.items()}
    L = {l["name"]: l for l in layers}

    def run(name, inp):
        l = L[name]
        return conv(inp, P[name][0], P[name][1], l["stride"], l["relu"])

    a0 = _r(x, bf16)
    a1 = _r(run("c1", a0), bf16)
    a2 = _r(run("c2", a1), bf16)
    a3 = _r(run("c3", a2), bf16)
    a4 = _r(run("c4", a3), bf16)
    a5 = _r(run("c5", a4), bf16)
    a6 = _r(run("c6", a5), bf16)
    u6 = _r(upsample2(a6, a3.shape[:3]), bf16)
    cat = np.concatenate([u6, a3], axis=-1)
    a7 = _r(run("c7", cat), bf16)
    pred = run("c8", a7)  # FP32 output on the GPU
    cache = dict(P=P, a0=a0, a1=a1, a2=a2, a3=a3, a4=a4, a5=a5, a6=a6, cat=cat, a7=a7, pred=pred)
    return pred, cache


def mse(pred, target):
    d = pred - target
    return float(np.mean(d * d)), 2.0 * d / d.size


def backward(cache, dpred, layers, bf16=False):
    """Gradients {name: (dW, db)} of the loss whose pred-gradient is dpred."""
    P = cache["P"]
    L = {l["name"]: l for l in layers}
    grads = {}

    def relu_mask(d, a):
        return np.where(a > 0, d, 0.0)

    def layer_back(name, dy, x_in, want_dx):
        l = L[name]
        dW, db = conv_wgrad(dy, x_in, l["stride"])
        grads[name] = (dW, db)
        if not want_dx:
            return None
        return conv_input_grad(dy, P[name][0], l["stride"], x_in.shape[:3])

    d8 = _r(dpred, bf16)
    d7 = _r(layer_back("c8", d8, cache["a7"], True), bf16)
    d7 = relu_mask(d7, cache["a7"])
    dcat = _r(layer_back("c7", d7, cache["cat"], True), bf16)
    c6 = cache["a6"].shape[-1]
    d6 = _r(upsample2_adjoint(dcat[..., :c6], cache["a6"].shape[:3]), bf16)
    d6 = relu_mask(d6, cache["a6"])
    d5 = relu_mask(_r(layer_back("c6", d6, cache["a5"], True), bf16), cache["a5"])
    d4 = relu_mask(_r(layer_back("c5", d5, cache["a4"], True), bf16), cache["a4"])
    # c3's output feeds c4 and the concatenation: the two gradients add (once
    # rounded, as the GPU accumulates into the stored concatenation gradient)
    d3 = _r(layer_back("c4", d4, cache["a3"], True) + dcat[..., c6:], bf16)
    d3 = relu_mask(d3, cache["a3"])
    d2 = relu_mask(_r(layer_back("c3", d3, cache["a2"], True), bf16), cache["a2"])
    d1 = relu_mask(_r(layer_back("c2", d2, cache["a1"], True), bf16), cache["a1"])
    layer_back("c1", d1, cache["a0"], False)
    return grads


def init_params(layers, seed=0):
    """He-normal weights (the last layer scaled by 0.1), zero biases."""
    rng = np.random.default_rng(seed)
    out = {}
    for i, l in enumerate(layers):
        std = np.sqrt(2.0 / (27 * l["cin"])) * (0.1 if i == len(layers) - 1 else 1.0)
        out[l["name"]] = (rng.standard_normal((l["cout"], 27, l["cin"])) * std, np.zeros(l["cout"]))
    return out
