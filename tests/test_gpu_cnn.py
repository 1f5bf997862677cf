"""CUDA kernels of the learned initial guess against the CPU oracle
(oracle/cnn_oracle.py), kernel by kernel and as a whole network (forward
output and every parameter gradient, BF16 rounding emulated in the oracle)."""
import ctypes as C

import numpy as np
import pytest

from oracle import cnn_oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module")
def env(cuda):
    import torch
    from voxeldvc_gb300 import _lib
    from voxeldvc_gb300.learned import seednet as S
    return torch, _lib, S


def bf(torch, a):
    """numpy (already BF16-representable) -> CUDA bfloat16 tensor, flat."""
    return torch.from_numpy(np.ascontiguousarray(a, np.float32).reshape(-1)).to("cuda").to(torch.bfloat16)


def host(t):
    return t.float().cpu().numpy().astype(np.float64)


def stream(torch):
    return torch.cuda.current_stream().cuda_stream


CONV_CASES = [  # (cin, n_out, stride, source grid (x, y, z))
    (2, 16, 1, (9, 7, 5)),
    (16, 32, 2, (9, 8, 7)),
    (32, 32, 1, (6, 5, 7)),
    (64, 16, 1, (5, 5, 5)),
    (16, 3, 1, (7, 6, 5)),
    (32, 80, 2, (5, 7, 9)),
    # beyond the mma.sync form (n_out > 80): the tcgen05 form only, several
    # 128-position tiles and a partial last tile
    (64, 128, 2, (17, 9, 11)),
    (128, 64, 1, (9, 10, 11)),
]


@pytest.mark.parametrize("cin,n_out,stride,src", CONV_CASES)
def test_conv_forward_input_grad_wgrad(env, cin, n_out, stride, src):
    torch, L, S = env
    lib = L.lib()
    rng = np.random.default_rng(cin * 7 + n_out)
    sx, sy, sz = src
    out = tuple((s - 1) // stride + 1 for s in src)
    x = O.bf16_round(rng.standard_normal((sz, sy, sx, cin)))
    W = rng.standard_normal((n_out, 27, cin)) * 0.2
    bvec = rng.standard_normal(n_out).astype(np.float32)
    Wr = O.bf16_round(W)
    ref = O.conv(x, Wr, bvec.astype(np.float64), stride, relu=True)
    # pack
    npad8, npad16, kpad8 = (n_out + 7) // 8 * 8, (n_out + 15) // 16 * 16, (cin + 7) // 8 * 8
    wt = torch.from_numpy(W.astype(np.float32).reshape(-1)).cuda()
    wf = torch.zeros(npad8 * (64 if cin == 2 else 27 * cin), dtype=torch.bfloat16, device="cuda")
    wb = torch.zeros(kpad8 * 27 * npad16, dtype=torch.bfloat16, device="cuda")
    L.check(lib.vdvc_cnn_pack_weights(wt.data_ptr(), n_out, cin, wf.data_ptr(), wb.data_ptr(), stream(torch)))
    xd = bf(torch, x)
    bd = torch.from_numpy(bvec).cuda()
    npos = out[0] * out[1] * out[2]
    y = torch.zeros(npos * n_out, dtype=torch.bfloat16, device="cuda")
    g = S.fwd_geom(out, src, stride)
    L.check(lib.vdvc_cnn_conv(xd.data_ptr(), cin, 0, cin, wf.data_ptr(), bd.data_ptr(), n_out, 1, y.data_ptr(), 0,
                              n_out, 0, 0, C.byref(g), stream(torch)))
    yh = host(y).reshape(ref.shape)
    assert np.allclose(yh, ref, rtol=8e-3, atol=8e-3 * np.abs(ref).max())

    # FP32 output, no activation
    yf = torch.zeros(npos * n_out, dtype=torch.float32, device="cuda")
    L.check(lib.vdvc_cnn_conv(xd.data_ptr(), cin, 0, cin, wf.data_ptr(), None, n_out, 0, yf.data_ptr(), 1, n_out, 0,
                              0, C.byref(g), stream(torch)))
    ref_lin = O.conv(x, Wr, None, stride, relu=False)
    assert rel(yf.cpu().numpy().reshape(ref.shape), ref_lin) < 1e-5

    # input gradient through the transposed weights and the adjoint geometry
    if cin != 2 and n_out <= 128:
        dy = O.bf16_round(rng.standard_normal(ref.shape))
        dyp = np.zeros(ref.shape[:3] + (npad16,))
        dyp[..., :n_out] = dy
        dx = torch.zeros(sx * sy * sz * cin, dtype=torch.bfloat16, device="cuda")
        gb = S.bwd_geom(src, out, stride)
        dypd = bf(torch, dyp)
        L.check(lib.vdvc_cnn_conv(dypd.data_ptr(), npad16, 0, npad16, wb.data_ptr(), None, cin, 0,
                                  dx.data_ptr(), 0, cin, 0, 0, C.byref(gb), stream(torch)))
        ref_dx = O.conv_input_grad(dy, Wr, stride, (sz, sy, sx))
        assert np.allclose(host(dx).reshape(ref_dx.shape), ref_dx, rtol=8e-3, atol=8e-3 * np.abs(ref_dx).max())

    # weight and bias gradients
    if True:  # every case: blocks of 32 x 64 channels tile the larger layers
        dy = O.bf16_round(rng.standard_normal(ref.shape))
        dw = torch.zeros(n_out * 27 * cin, dtype=torch.float32, device="cuda")
        db = torch.zeros(n_out, dtype=torch.float32, device="cuda")
        nb = lib.vdvc_cnn_wgrad_workspace_bytes(n_out, cin)
        ws = torch.empty(nb, dtype=torch.uint8, device="cuda")
        dyd = bf(torch, dy)
        L.check(lib.vdvc_cnn_conv_wgrad(dyd.data_ptr(), n_out, 0, n_out, xd.data_ptr(), cin, 0, cin, C.byref(g),
                                        dw.data_ptr(), 0, ws.data_ptr(), nb, stream(torch)))
        L.check(lib.vdvc_cnn_bias_grad(dyd.data_ptr(), n_out, 0, n_out, npos, db.data_ptr(), 0, ws.data_ptr(), nb,
                                       stream(torch)))
        ref_dw, ref_db = O.conv_wgrad(dy, x, stride)
        assert rel(dw.cpu().numpy().reshape(ref_dw.shape), ref_dw) < 1e-5
        assert rel(db.cpu().numpy(), ref_db) < 1e-5
        # accumulate mode adds
        L.check(lib.vdvc_cnn_conv_wgrad(dyd.data_ptr(), n_out, 0, n_out, xd.data_ptr(), cin, 0, cin, C.byref(g),
                                        dw.data_ptr(), 1, ws.data_ptr(), nb, stream(torch)))
        assert rel(dw.cpu().numpy().reshape(ref_dw.shape), 2 * ref_dw) < 1e-5


@pytest.mark.parametrize("cin,n_out,stride,src", [(64, 64, 1, (33, 33, 65)), (32, 32, 2, (65, 65, 129)),
                                                  (128, 128, 1, (33, 17, 49))])
def test_conv_persistent_many_bricks(env, cin, n_out, stride, src):
    """More output bricks than resident CTAs (2 per SM): every CTA of the
    persistent form walks several bricks through its stage ring, the two
    TMEM accumulators alternating -- against the oracle."""
    torch, L, S = env
    lib = L.lib()
    rng = np.random.default_rng(cin + n_out + stride)
    sx, sy, sz = src
    out = tuple((s - 1) // stride + 1 for s in src)
    nbricks = -(-out[0] // 8) * -(-out[1] // 4) * -(-out[2] // 4)
    assert nbricks > 2 * torch.cuda.get_device_properties(0).multi_processor_count
    x = O.bf16_round(rng.standard_normal((sz, sy, sx, cin)))
    W = rng.standard_normal((n_out, 27, cin)) * 0.1
    bvec = rng.standard_normal(n_out).astype(np.float32)
    ref = O.conv(x, O.bf16_round(W), bvec.astype(np.float64), stride, relu=True)
    wf = torch.zeros((n_out + 7) // 8 * 8 * 27 * cin, dtype=torch.bfloat16, device="cuda")
    wt = torch.from_numpy(W.astype(np.float32).reshape(-1)).cuda()
    L.check(lib.vdvc_cnn_pack_weights(wt.data_ptr(), n_out, cin, wf.data_ptr(), None, stream(torch)))
    xd, bd = bf(torch, x), torch.from_numpy(bvec).cuda()
    y = torch.zeros(out[0] * out[1] * out[2] * n_out, dtype=torch.bfloat16, device="cuda")
    g = S.fwd_geom(out, src, stride)
    L.check(lib.vdvc_cnn_conv(xd.data_ptr(), cin, 0, cin, wf.data_ptr(), bd.data_ptr(), n_out, 1, y.data_ptr(), 0,
                              n_out, 0, 0, C.byref(g), stream(torch)))
    L.check(lib.vdvc_cnn_status(stream(torch)))
    yh = host(y).reshape(ref.shape)
    assert np.allclose(yh, ref, rtol=8e-3, atol=8e-3 * np.abs(ref).max())


@pytest.mark.parametrize("cin,n_out,stride,scs,scoff", [(64, 64, 1, 128, 64), (32, 64, 2, 96, 32),
                                                        (256, 64, 1, 256, 0), (128, 128, 2, 256, 128)])
def test_conv_channel_slices_and_accumulate(env, cin, n_out, stride, scs, scoff):
    """A channel slice of a wider source (the decoder's concatenated
    buffers) into a channel slice of a wider output, written and then added
    on top (accumulate); grids that are not multiples of the 8 x 4 x 4
    output bricks."""
    torch, L, S = env
    lib = L.lib()
    rng = np.random.default_rng(cin + scs + stride)
    src = (11, 6, 9)
    sx, sy, sz = src
    out = tuple((s - 1) // stride + 1 for s in src)
    xw = O.bf16_round(rng.standard_normal((sz, sy, sx, scs)))
    x = xw[..., scoff:scoff + cin]
    W = rng.standard_normal((n_out, 27, cin)) * 0.1
    Wr = O.bf16_round(W)
    bvec = rng.standard_normal(n_out).astype(np.float32)
    ref = O.conv(x, Wr, bvec.astype(np.float64), stride, relu=True)
    npad8, npad16 = (n_out + 7) // 8 * 8, (n_out + 15) // 16 * 16
    wf = torch.zeros(npad8 * 27 * cin, dtype=torch.bfloat16, device="cuda")
    wb = torch.zeros((cin + 7) // 8 * 8 * 27 * npad16, dtype=torch.bfloat16, device="cuda")
    wt = torch.from_numpy(W.astype(np.float32).reshape(-1)).cuda()
    L.check(lib.vdvc_cnn_pack_weights(wt.data_ptr(), n_out, cin, wf.data_ptr(), wb.data_ptr(), stream(torch)))
    ocs, ocoff = n_out + 16, 8
    npos = out[0] * out[1] * out[2]
    base = O.bf16_round(rng.standard_normal((npos, ocs)))
    y = bf(torch, base)
    g = S.fwd_geom(out, src, stride)
    xd, bd = bf(torch, xw), torch.from_numpy(bvec).cuda()  # held: the launches are asynchronous
    L.check(lib.vdvc_cnn_conv(xd.data_ptr(), scs, scoff, cin, wf.data_ptr(), bd.data_ptr(), n_out, 1, y.data_ptr(), 0,
                              ocs, ocoff, 0, C.byref(g), stream(torch)))
    yh = host(y).reshape(npos, ocs)
    r2 = ref.reshape(npos, n_out)
    tol = 8e-3 * np.abs(r2).max()
    assert np.allclose(yh[:, ocoff:ocoff + n_out], r2, rtol=8e-3, atol=tol)
    # channels outside the slice untouched
    assert np.array_equal(yh[:, :ocoff], base[:, :ocoff])
    assert np.array_equal(yh[:, ocoff + n_out:], base[:, ocoff + n_out:])
    L.check(lib.vdvc_cnn_conv(xd.data_ptr(), scs, scoff, cin, wf.data_ptr(), bd.data_ptr(), n_out, 1, y.data_ptr(), 0,
                              ocs, ocoff, 1, C.byref(g), stream(torch)))
    yh2 = host(y).reshape(npos, ocs)
    assert np.allclose(yh2[:, ocoff:ocoff + n_out], 2 * r2, rtol=1.6e-2, atol=2 * tol)
    assert np.array_equal(yh2[:, :ocoff], base[:, :ocoff])
    L.check(lib.vdvc_cnn_status(stream(torch)))


@pytest.mark.parametrize("m,n", [((3, 4, 5), (5, 7, 9)), ((3, 3, 3), (6, 6, 6))])
def test_upsample(env, m, n):
    torch, L, S = env
    lib = L.lib()
    rng = np.random.default_rng(1)
    c = O.bf16_round(rng.standard_normal((m[2], m[1], m[0], 4)))
    f = torch.zeros(n[0] * n[1] * n[2] * 8, dtype=torch.bfloat16, device="cuda")
    cd = bf(torch, c)
    L.check(lib.vdvc_cnn_upsample2(cd.data_ptr(), 4, 0, *m, f.data_ptr(), 8, 4, *n, 4, stream(torch)))
    ref = O.upsample2(c, (n[2], n[1], n[0]))
    fh = host(f).reshape(n[2], n[1], n[0], 8)
    assert np.allclose(fh[..., 4:], ref, rtol=8e-3, atol=1e-2)
    assert np.all(fh[..., :4] == 0)
    df = O.bf16_round(rng.standard_normal((n[2], n[1], n[0], 4)))
    dc = torch.zeros(m[0] * m[1] * m[2] * 4, dtype=torch.bfloat16, device="cuda")
    dfd = bf(torch, df)
    L.check(lib.vdvc_cnn_upsample2_bwd(dfd.data_ptr(), 4, 0, *n, dc.data_ptr(), 4, 0, *m, 4, stream(torch)))
    ref_dc = O.upsample2_adjoint(df, (m[2], m[1], m[0]))
    assert np.allclose(host(dc).reshape(ref_dc.shape), ref_dc, rtol=8e-3, atol=2e-2)
    # 16 channels at 8-channel-aligned strides and offsets (the 16-byte
    # form) against the oracle and, bit for bit, against the per-channel
    # form (an offset of 2 channels keeps that one)
    c16 = O.bf16_round(rng.standard_normal((m[2], m[1], m[0], 24)))
    c16d = bf(torch, c16)
    fa = torch.zeros(n[0] * n[1] * n[2] * 32, dtype=torch.bfloat16, device="cuda")
    fb = torch.zeros(n[0] * n[1] * n[2] * 32, dtype=torch.bfloat16, device="cuda")
    L.check(lib.vdvc_cnn_upsample2(c16d.data_ptr(), 24, 8, *m, fa.data_ptr(), 32, 8, *n, 16, stream(torch)))
    L.check(lib.vdvc_cnn_upsample2(c16d.data_ptr(), 24, 8, *m, fb.data_ptr(), 32, 2, *n, 16, stream(torch)))
    ref16 = O.upsample2(c16[..., 8:24], (n[2], n[1], n[0]))
    fa4 = fa.view(n[2], n[1], n[0], 32)
    assert np.allclose(host(fa4[..., 8:24]), ref16, rtol=8e-3, atol=1e-2)
    assert torch.equal(fa4[..., 8:24], fb.view(n[2], n[1], n[0], 32)[..., 2:18])
    assert not torch.any(fa4[..., :8]) and not torch.any(fa4[..., 24:])


def test_pool_input_mse_adam_seed(env):
    torch, L, S = env
    lib = L.lib()
    rng = np.random.default_rng(2)
    nx, ny, nz = 17, 13, 9
    f = rng.random((nz, ny, nx)).astype(np.float32)
    g = rng.random((nz, ny, nx)).astype(np.float32)
    ms = np.array([0.4, 0.3, 0.6, 0.2])
    gx, gy, gz = (nx - 1) // 4 + 1, (ny - 1) // 4 + 1, (nz - 1) // 4 + 1
    out = torch.zeros(gx * gy * gz * 2, dtype=torch.bfloat16, device="cuda")
    # device copies are held in names: a temporary's memory may be reused
    # before the kernel runs
    fd, gd_img = torch.from_numpy(f.reshape(-1)).cuda(), torch.from_numpy(g.reshape(-1)).cuda()
    L.check(lib.vdvc_cnn_pool_input(fd.data_ptr(), gd_img.data_ptr(), nx, ny, nz, ms.ctypes.data_as(L.pd),
                                    out.data_ptr(), stream(torch)))
    ref = O.pool_input(f, g, ms)
    assert np.allclose(host(out).reshape(ref.shape), ref, rtol=8e-3, atol=1e-2)

    # mse and its gradient
    npos = 50
    pred = rng.standard_normal((npos, 8)).astype(np.float32)
    tgt = rng.standard_normal((npos, 3)).astype(np.float32)
    loss = torch.zeros(1, dtype=torch.float64, device="cuda")
    dp = torch.zeros(npos * 16, dtype=torch.bfloat16, device="cuda")
    ws = torch.empty(1 << 16, dtype=torch.uint8, device="cuda")
    pd_, td = torch.from_numpy(pred.reshape(-1)).cuda(), torch.from_numpy(tgt.reshape(-1)).cuda()
    L.check(lib.vdvc_cnn_mse(pd_.data_ptr(), 8, td.data_ptr(), npos, loss.data_ptr(), dp.data_ptr(), 16, 2.0,
                             ws.data_ptr(), ws.numel(), stream(torch)))
    l_ref, d_ref = O.mse(pred[:, :3].astype(np.float64), tgt.astype(np.float64))
    assert abs(loss.item() - l_ref) < 1e-12 * max(1, l_ref)
    dph = host(dp).reshape(npos, 16)
    assert np.allclose(dph[:, :3], 2.0 * d_ref, rtol=8e-3) and np.all(dph[:, 3:] == 0)

    # Adam
    n = 1000
    w0 = rng.standard_normal(n).astype(np.float32)
    gr = rng.standard_normal(n).astype(np.float32)
    w, m, v = (torch.from_numpy(a.copy()).cuda() for a in (w0, np.zeros(n, np.float32), np.zeros(n, np.float32)))
    gd = torch.from_numpy(gr).cuda()
    for step in (1, 2):
        L.check(lib.vdvc_cnn_adam(w.data_ptr(), gd.data_ptr(), m.data_ptr(), v.data_ptr(), n, 1e-2, 0.9, 0.999, 1e-8,
                                  step, stream(torch)))
    mr, vr, wr = np.zeros(n), np.zeros(n), w0.astype(np.float64)
    for step in (1, 2):
        mr = 0.9 * mr + 0.1 * gr
        vr = 0.999 * vr + 0.001 * gr.astype(np.float64) ** 2
        wr = wr - 1e-2 * (mr / (1 - 0.9 ** step)) / (np.sqrt(vr / (1 - 0.999 ** step)) + 1e-8)
    assert np.allclose(w.cpu().numpy(), wr, rtol=1e-5, atol=1e-6)

    # nodal seed: trilinear resampling of the stride-8 output at node * h
    px, py, pz = 5, 4, 3
    pr = rng.standard_normal((pz, py, px, 8)).astype(np.float32)
    h, Nx, Ny, Nz = 4, 8, 6, 4
    U = torch.zeros(3 * (Nx + 1) * (Ny + 1) * (Nz + 1), dtype=torch.float64, device="cuda")
    prd = torch.from_numpy(pr.reshape(-1)).cuda()
    L.check(lib.vdvc_cnn_seed_nodes(prd.data_ptr(), 8, px, py, pz, h, Nx, Ny, Nz, U.data_ptr(), stream(torch)))
    from scipy.ndimage import map_coordinates
    k, j, i = np.meshgrid(np.arange(Nz + 1), np.arange(Ny + 1), np.arange(Nx + 1), indexing="ij")
    coords = np.stack([k * h / 8.0, j * h / 8.0, i * h / 8.0]).reshape(3, -1)
    ref = np.stack([map_coordinates(pr[..., c].astype(np.float64), coords, order=1, mode="nearest")
                    for c in range(3)], axis=1).reshape(-1)
    assert np.allclose(U.cpu().numpy(), ref, atol=1e-5)


def test_input_moments_device_pool_and_mirror(env):
    """The one-pass image moments against float64 sums; pooling with the
    statistics taken on the device equals pooling with the same statistics
    computed on the host (bit for bit); mirroring the pooled grid equals
    pooling the mirrored pair where the pooling grid is symmetric (up to the
    FP32 summation order of a window)."""
    torch, L, S = env
    lib = L.lib()
    rng = np.random.default_rng(9)
    nx, ny, nz = 21, 13, 9  # (n - 1) % 4 == 0 along every axis
    f = (rng.random((nz, ny, nx)) * 3 + 1).astype(np.float32)
    g = (rng.random((nz, ny, nx)) * 2 - 0.5).astype(np.float32)
    fd, gd = torch.from_numpy(f.reshape(-1)).cuda(), torch.from_numpy(g.reshape(-1)).cuda()
    n = f.size
    sums = torch.zeros(4, dtype=torch.float64, device="cuda")
    ws = torch.empty(1 << 16, dtype=torch.uint8, device="cuda")
    L.check(lib.vdvc_cnn_input_moments(fd.data_ptr(), gd.data_ptr(), n, sums.data_ptr(), ws.data_ptr(), ws.numel(),
                                       stream(torch)))
    hs = sums.cpu().numpy()
    f64, g64 = f.astype(np.float64), g.astype(np.float64)
    ref = np.array([f64.sum(), (f64 * f64).sum(), g64.sum(), (g64 * g64).sum()])
    assert np.allclose(hs, ref, rtol=1e-6)
    # an unaligned tail (no float4 path) gives the same sums
    L.check(lib.vdvc_cnn_input_moments(fd[1:].data_ptr(), gd[1:].data_ptr(), n - 1, sums.data_ptr(), ws.data_ptr(),
                                       ws.numel(), stream(torch)))
    ref1 = np.array([f64.reshape(-1)[1:].sum(), (f64.reshape(-1)[1:] ** 2).sum(), g64.reshape(-1)[1:].sum(),
                     (g64.reshape(-1)[1:] ** 2).sum()])
    assert np.allclose(sums.cpu().numpy(), ref1, rtol=1e-6)
    mf, mg = hs[0] / n, hs[2] / n
    ms = np.array([mf, np.sqrt(hs[1] / n - mf * mf), mg, np.sqrt(hs[3] / n - mg * mg)])
    sums.copy_(torch.from_numpy(hs))
    gx, gy, gz = (nx - 1) // 4 + 1, (ny - 1) // 4 + 1, (nz - 1) // 4 + 1
    x0 = torch.zeros(gx * gy * gz * 2, dtype=torch.bfloat16, device="cuda")
    for flip in range(8):
        a = torch.zeros_like(x0)
        b = torch.zeros_like(x0)
        L.check(lib.vdvc_cnn_pool_input_dev(fd.data_ptr(), gd.data_ptr(), nx, ny, nz, sums.data_ptr(), flip,
                                            a.data_ptr(), stream(torch)))
        L.check(lib.vdvc_cnn_pool_input_mirrored(fd.data_ptr(), gd.data_ptr(), nx, ny, nz, ms.ctypes.data_as(L.pd),
                                                 flip, b.data_ptr(), stream(torch)))
        assert torch.equal(a, b), flip
        if flip == 0:
            x0.copy_(a)
        else:
            m = torch.zeros_like(x0)
            L.check(lib.vdvc_cnn_mirror_input(x0.data_ptr(), gx, gy, gz, flip, m.data_ptr(), stream(torch)))
            # the same windows summed in the mirrored FP32 order: an element
            # may round to the neighbouring BF16 value
            mf32, bf32 = m.float(), b.float()
            assert torch.allclose(mf32, bf32, rtol=2.0 ** -7, atol=1e-30), flip
            assert (mf32 != bf32).float().mean().item() < 0.01, flip
    with pytest.raises(Exception):
        L.check(lib.vdvc_cnn_mirror_input(x0.data_ptr(), gx, gy, gz, 1, x0.data_ptr(), stream(torch)))


def test_mirrored_pool_and_seed(env):
    """The mirrored input pooling equals the pooling of the mirrored images,
    and a mirrored pass's output accumulated into the seed equals the
    unmirrored field it stands for (averaging two equal predictions gives
    the prediction back)."""
    torch, L, S = env
    lib = L.lib()
    rng = np.random.default_rng(4)
    nx, ny, nz = 17, 13, 9
    f = rng.random((nz, ny, nx)).astype(np.float32)
    g = rng.random((nz, ny, nx)).astype(np.float32)
    ms = np.array([0.4, 0.3, 0.6, 0.2])
    gx, gy, gz = (nx - 1) // 4 + 1, (ny - 1) // 4 + 1, (nz - 1) // 4 + 1
    fd, gd = torch.from_numpy(f.reshape(-1)).cuda(), torch.from_numpy(g.reshape(-1)).cuda()
    for flip in (1, 2, 3, 5, 7):
        axes = tuple(2 - k for k in range(3) if (flip >> k) & 1)  # numpy axes of x, y, z in (z, y, x)
        fm = torch.from_numpy(np.ascontiguousarray(np.flip(f, axes)).reshape(-1)).cuda()
        gm = torch.from_numpy(np.ascontiguousarray(np.flip(g, axes)).reshape(-1)).cuda()
        a = torch.zeros(gx * gy * gz * 2, dtype=torch.bfloat16, device="cuda")
        b = torch.zeros_like(a)
        L.check(lib.vdvc_cnn_pool_input_mirrored(fd.data_ptr(), gd.data_ptr(), nx, ny, nz, ms.ctypes.data_as(L.pd),
                                                 flip, a.data_ptr(), stream(torch)))
        L.check(lib.vdvc_cnn_pool_input(fm.data_ptr(), gm.data_ptr(), nx, ny, nz, ms.ctypes.data_as(L.pd),
                                        b.data_ptr(), stream(torch)))
        assert torch.equal(a, b), flip
    # seed: pred0 on the output grid of a 33 x 25 x 17 volume meshed at h = 4
    px, py, pz = 5, 4, 3
    h, Nx, Ny, Nz = 4, 8, 6, 4
    pr = rng.standard_normal((pz, py, px, 8)).astype(np.float32)
    n = 3 * (Nx + 1) * (Ny + 1) * (Nz + 1)
    U1 = torch.zeros(n, dtype=torch.float64, device="cuda")
    U2 = torch.zeros(n, dtype=torch.float64, device="cuda")
    p0 = torch.from_numpy(pr.reshape(-1)).cuda()
    L.check(lib.vdvc_cnn_seed_nodes(p0.data_ptr(), 8, px, py, pz, h, Nx, Ny, Nz, U1.data_ptr(), stream(torch)))
    for flip in (1, 2, 3, 4, 7):
        axes = tuple(2 - k for k in range(3) if (flip >> k) & 1)
        pm = np.flip(pr, axes).copy()
        for k in range(3):
            if (flip >> k) & 1:
                pm[..., k] = -pm[..., k]
        pmd = torch.from_numpy(pm.reshape(-1)).cuda()
        L.check(lib.vdvc_cnn_seed_nodes_acc(p0.data_ptr(), 8, px, py, pz, h, Nx, Ny, Nz, 0, 0.5, 0, U2.data_ptr(),
                                            stream(torch)))
        L.check(lib.vdvc_cnn_seed_nodes_acc(pmd.data_ptr(), 8, px, py, pz, h, Nx, Ny, Nz, flip, 0.5, 1,
                                            U2.data_ptr(), stream(torch)))
        assert torch.allclose(U1, U2, atol=1e-6), flip
    # a mesh that does not span the output grid cannot be mirrored
    with pytest.raises(Exception):
        L.check(lib.vdvc_cnn_seed_nodes_acc(p0.data_ptr(), 8, px, py, pz, h, Nx - 1, Ny, Nz, 1, 1.0, 0,
                                            U2.data_ptr(), stream(torch)))


def test_network_forward_and_gradients(env):
    """The whole network on the GPU vs the oracle with BF16 emulation."""
    torch, L, S = env
    from voxeldvc_gb300.learned.arch import LAYERS, grids
    rng = np.random.default_rng(11)
    params = O.init_params(LAYERS, seed=3)
    params = {k: (W, rng.standard_normal(b.shape) * 0.05) for k, (W, b) in params.items()}
    net = S.SeedNet(params)
    G = (17, 13, 9)
    G, n, _, _ = grids(G)
    x = O.bf16_round(rng.standard_normal((G[2], G[1], G[0], 2)))
    target = rng.standard_normal((n[2], n[1], n[0], 3)).astype(np.float32)
    b = net.buffers(G)
    b["x"].copy_(bf(torch, x))
    pred = net.forward(G)
    tg = torch.from_numpy(target.reshape(-1)).cuda()
    loss = net.loss(G, tg)
    net.backward(G)
    torch.cuda.synchronize()
    pnp = {k: (v[0].astype(np.float32).astype(np.float64), v[1].astype(np.float32).astype(np.float64))
           for k, v in params.items()}
    ref_pred, cache = O.forward(pnp, x, LAYERS, bf16=True)
    gp = pred.cpu().numpy().reshape(n[2], n[1], n[0], 8)[..., :3]
    assert rel(gp, ref_pred) < 1e-2
    l_ref, d_ref = O.mse(gp.astype(np.float64), target.astype(np.float64))
    assert abs(loss.item() - l_ref) < 1e-6 * l_ref
    grads = O.backward(cache, d_ref, LAYERS, bf16=True)
    gg = net.grads_numpy()
    for name in grads:
        assert rel(gg[name][0], grads[name][0]) < 3e-2, name
        assert rel(gg[name][1], grads[name][1]) < 3e-2, name
