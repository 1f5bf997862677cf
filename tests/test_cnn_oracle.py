"""The network oracle pinned on the CPU: its backward pass against finite
differences, its convolution adjoint against the forward operator, and its
upsampling adjoint (the oracle is the checker of the CUDA network kernels)."""
import numpy as np
import pytest

from oracle import cnn_oracle as O
from voxeldvc_gb300.learned.arch import LAYERS, grids


def test_bf16_round():
    x = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, -2.5, 0.0])
    assert np.array_equal(O.bf16_round(x), [1.0, 1.0, 1.0 + 2.0 ** -6, -2.5, 0.0])


@pytest.mark.parametrize("stride", [1, 2])
def test_conv_adjoint(stride):
    rng = np.random.default_rng(stride)
    x = rng.standard_normal((5, 6, 7, 3))
    W = rng.standard_normal((4, 27, 3))
    y = O.conv(x, W, None, stride, relu=False)
    dy = rng.standard_normal(y.shape)
    dx = O.conv_input_grad(dy, W, stride, x.shape[:3])
    assert abs(np.sum(y * dy) - np.sum(x * dx)) < 1e-9 * np.abs(y * dy).sum()
    dW, db = O.conv_wgrad(dy, x, stride)
    # <dy, conv(x, W)> is linear in W: its gradient is dW
    V = rng.standard_normal(W.shape)
    assert abs(np.sum(O.conv(x, V, None, stride, False) * dy) - np.sum(V * dW)) < 1e-9 * np.abs(dW).sum() * 10
    assert np.allclose(db, dy.reshape(-1, 4).sum(0))


def test_conv_matches_direct_loop():
    rng = np.random.default_rng(3)
    x = rng.standard_normal((4, 5, 5, 2))
    W = rng.standard_normal((3, 27, 2))
    y = O.conv(x, W, None, 2, relu=False)
    ref = np.zeros_like(y)
    for z in range(y.shape[0]):
        for yy in range(y.shape[1]):
            for xx in range(y.shape[2]):
                for t in range(27):
                    qx, qy, qz = 2 * xx - 1 + t % 3, 2 * yy - 1 + (t // 3) % 3, 2 * z - 1 + t // 9
                    if 0 <= qx < 5 and 0 <= qy < 5 and 0 <= qz < 4:
                        ref[z, yy, xx] += W[:, t, :] @ x[qz, qy, qx]
    assert np.allclose(y, ref, atol=1e-12)


@pytest.mark.parametrize("n,m", [(5, 3), (6, 3), (9, 5)])
def test_upsample_adjoint(n, m):
    rng = np.random.default_rng(n)
    c = rng.standard_normal((m, m, m, 2))
    f = O.upsample2(c, (n, n, n))
    df = rng.standard_normal(f.shape)
    dc = O.upsample2_adjoint(df, (m, m, m))
    assert abs(np.sum(f * df) - np.sum(c * dc)) < 1e-10 * np.abs(f * df).sum()


def test_network_gradient_finite_differences():
    G, n, m, _ = grids((9, 9, 9))
    rng = np.random.default_rng(7)
    params = O.init_params(LAYERS, seed=1)
    # non-zero biases exercise the bias gradients too
    params = {k: (W, rng.standard_normal(b.shape) * 0.1) for k, (W, b) in params.items()}
    x = rng.standard_normal(tuple(reversed(G)) + (2,))
    target = rng.standard_normal(tuple(reversed(n)) + (3,))

    def loss(p):
        pred, _ = O.forward(p, x, LAYERS)
        return O.mse(pred, target)[0]

    pred, cache = O.forward(params, x, LAYERS)
    _, dpred = O.mse(pred, target)
    grads = O.backward(cache, dpred, LAYERS)
    for trial in range(3):
        V = {k: (rng.standard_normal(W.shape), rng.standard_normal(b.shape)) for k, (W, b) in params.items()}
        eps = 1e-7  # small enough that no ReLU kink is crossed
        pp = {k: (W + eps * V[k][0], b + eps * V[k][1]) for k, (W, b) in params.items()}
        pm = {k: (W - eps * V[k][0], b - eps * V[k][1]) for k, (W, b) in params.items()}
        fd = (loss(pp) - loss(pm)) / (2 * eps)
        an = sum(np.sum(grads[k][0] * V[k][0]) + np.sum(grads[k][1] * V[k][1]) for k in params)
        assert abs(fd - an) <= 1e-5 * max(1.0, abs(an)), (fd, an)


def test_pool_input_constant_and_shape():
    f = np.full((9, 10, 13), 3.0)
    g = np.full((9, 10, 13), 5.0)
    out = O.pool_input(f, g, (1.0, 2.0, 1.0, 4.0))
    assert out.shape == (3, 3, 4, 2)
    assert np.allclose(out[..., 0], 1.0) and np.allclose(out[..., 1], 1.0)


def test_arch_layout_and_grids():
    from voxeldvc_gb300.learned.arch import param_layout, grids, input_grid, LAYERS
    layout, total = param_layout()
    assert [l[0] for l in layout] == [l["name"] for l in LAYERS]
    off = 0
    for (name, wo, ws, bo, n_out, cin), l in zip(layout, LAYERS):
        assert wo == off and ws == n_out * 27 * cin and bo == wo + ws
        off = bo + n_out
    assert total == off
    # 513^3 voxels: input grid 129, output (node grid of h = 8) 65, then 33, 17
    assert input_grid((513, 513, 513)) == (129, 129, 129)
    assert grids((129, 129, 129)) == ((129, 129, 129), (65, 65, 65), (33, 33, 33), (17, 17, 17))
    assert grids((65, 40, 9))[1:] == ((33, 20, 5), (17, 10, 3), (9, 5, 2))
    # the configuration's size: about 2M parameters
    assert 2.0e6 < total < 2.5e6
