"""Host side of the learned initial guess: the network of `arch` run on the
GPU through the kernels of include/vdvc_cnn.h (forward, backward, Adam),
plus loading and saving of its FP32 master weights.

Device memory is held in torch tensors (plumbing only: every operation on
them is one of this package's kernels).  The FP32 master weights live in one
flat vector, laid out by `arch.param_layout()`, so the optimiser is a single
launch; after every update the BF16 copies each convolution reads are
repacked (forward layout, and the transposed layout of the input gradient).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .. import _device as D
from .. import _lib
from .arch import LAYERS, LAYER, grids, param_layout, input_grid, OUT_STRIDE

WEIGHTS_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "seed_net.npz")


def _geom(out_grid, src_grid, a, b, c, d):
    g = _lib.ConvGeom()
    g.nx, g.ny, g.nz = out_grid
    g.sx, g.sy, g.sz = src_grid
    g.a, g.b, g.c, g.d = a, b, c, d
    return g


def fwd_geom(out_grid, src_grid, stride):
    return _geom(out_grid, src_grid, stride, -1, 1, 1)


def bwd_geom(out_grid, src_grid, stride):
    """Input gradient of a stride-`stride` convolution: out_grid is the
    forward source grid, src_grid the forward output grid."""
    return _geom(out_grid, src_grid, 1, 1, -1, stride)


def _npos(grid):
    return int(grid[0]) * int(grid[1]) * int(grid[2])


def _pad(n, k):
    return (n + k - 1) // k * k


class SeedNet:
    """The network with its parameters on the current CUDA device."""

    def __init__(self, params=None, seed=0):
        torch = D.torch()
        self.layout, self.nparam = param_layout()
        flat = np.zeros(self.nparam, np.float32)
        if params is None:
            rng = np.random.default_rng(seed)
            params = {}
            for i, l in enumerate(LAYERS):
                std = np.sqrt(2.0 / (27 * l["cin"])) * (0.1 if i == len(LAYERS) - 1 else 1.0)
                params[l["name"]] = (rng.standard_normal((l["cout"], 27, l["cin"])) * std, np.zeros(l["cout"]))
        for name, wo, ws, bo, n_out, cin in self.layout:
            W, b = params[name]
            W = np.asarray(W, np.float32)
            if W.shape != (n_out, 27, cin):
                raise ValueError(f"{name}: weights of shape {W.shape}, expected {(n_out, 27, cin)}")
            flat[wo:wo + ws] = W.reshape(-1)
            flat[bo:bo + n_out] = np.asarray(b, np.float32).reshape(-1)
        self.theta = D.to_device(flat)
        self.grad = torch.zeros_like(self.theta)
        self.m = torch.zeros_like(self.theta)
        self.v = torch.zeros_like(self.theta)
        self.step_count = 0
        self.wf, self.wb = {}, {}
        for name, wo, ws, bo, n_out, cin in self.layout:
            nf = _pad(n_out, 8) * (64 if cin == 2 else 27 * cin)
            self.wf[name] = torch.zeros(nf, dtype=torch.bfloat16, device=D.device())
            if cin != 2:  # the first layer needs no input gradient
                self.wb[name] = torch.zeros(_pad(cin, 8) * 27 * _pad(n_out, 16), dtype=torch.bfloat16,
                                            device=D.device())
        self._bufs = {}
        self.pack()

    # ---- parameters ------------------------------------------------------------

    def _wptr(self, name, grad=False):
        base = (self.grad if grad else self.theta).data_ptr()
        for n, wo, ws, bo, n_out, cin in self.layout:
            if n == name:
                return base + 4 * wo, base + 4 * bo
        raise KeyError(name)

    def pack(self):
        L = _lib.lib()
        for name, wo, ws, bo, n_out, cin in self.layout:
            wptr, _ = self._wptr(name)
            wb = self.wb.get(name)
            _lib.check(L.vdvc_cnn_pack_weights(wptr, n_out, cin, self.wf[name].data_ptr(),
                                               wb.data_ptr() if wb is not None else None, D.stream()),
                       "cnn_pack_weights")

    def params_numpy(self):
        flat = self.theta.cpu().numpy()
        out = {}
        for name, wo, ws, bo, n_out, cin in self.layout:
            out[name] = (flat[wo:wo + ws].reshape(n_out, 27, cin).copy(), flat[bo:bo + n_out].copy())
        return out

    def grads_numpy(self):
        flat = self.grad.cpu().numpy()
        out = {}
        for name, wo, ws, bo, n_out, cin in self.layout:
            out[name] = (flat[wo:wo + ws].reshape(n_out, 27, cin).copy(), flat[bo:bo + n_out].copy())
        return out

    def save(self, path, **meta):
        """Weights as BF16 bit patterns (the convolutions read BF16 copies of
        them, so nothing is lost for inference), biases FP32."""
        p = self.params_numpy()
        arrays = {f"{k}_W16": _to_bf16_bits(v[0]) for k, v in p.items()}
        arrays.update({f"{k}_b": v[1] for k, v in p.items()})
        arrays.update({f"meta_{k}": np.asarray(v) for k, v in meta.items()})
        np.savez_compressed(path, **arrays)

    @classmethod
    def load(cls, path=WEIGHTS_PATH):
        z = np.load(path)
        params = {}
        for l in LAYERS:
            n = l["name"]
            W = _from_bf16_bits(z[f"{n}_W16"]) if f"{n}_W16" in z.files else z[f"{n}_W"]
            params[n] = (W, z[f"{n}_b"])
        net = cls(params)
        net.meta = {k[5:]: z[k] for k in z.files if k.startswith("meta_")}
        return net

    # ---- buffers -----------------------------------------------------------------

    # Channels-last BF16 buffers per grid level (0: input grid; 1: the output
    # grid, stride 8 voxels; 2, 3: coarser), and gradient buffers of the
    # same shapes.  Concatenations are one buffer: cat3 = [up(e4b) | e3b] at
    # level 2, cat2 = [up(d3) | e2b] at level 1; the encoder writes its skip
    # output straight into the upper channels.
    _ACT = (("x", 0, 2), ("e1", 0, 32), ("e2a", 1, 64), ("cat2", 1, 128), ("e3a", 2, 128), ("cat3", 2, 256),
            ("e4a", 3, 128), ("e4b", 3, 128), ("d3", 2, 64), ("d2", 1, 32))
    _GRAD = (("dp", 1, 16), ("dd2", 1, 32), ("dcat2", 1, 128), ("dd3", 2, 64), ("dcat3", 2, 256),
             ("de4b", 3, 128), ("de4a", 3, 128), ("de3a", 2, 128), ("de2a", 1, 64), ("de1", 0, 32))

    def buffers(self, G, train=True, slot=0):
        """Activation (and, with train, gradient) buffers for input grid G
        (cached).  Inference passes that run concurrently (the mirrored
        passes of predict_nodes) use separate slots."""
        G = tuple(int(v) for v in G)
        if slot:
            key = (G, False, slot)
            if key not in self._bufs:
                self._bufs[key] = self._alloc(G, False)
            return self._bufs[key]
        if (G, True) in self._bufs:
            return self._bufs[(G, True)]
        if not train and (G, False) in self._bufs:
            return self._bufs[(G, False)]
        b = self._alloc(G, train)
        self._bufs[(G, bool(train))] = b
        return b

    def _alloc(self, G, train):
        torch = D.torch()
        lv = grids(G)
        bf = lambda level, c: torch.zeros(_npos(lv[level]) * c, dtype=torch.bfloat16, device=D.device())
        b = dict(G=G, lv=lv)
        for name, level, c in self._ACT:
            b[name] = bf(level, c)
        b["pred"] = torch.zeros(_npos(lv[1]) * 8, dtype=torch.float32, device=D.device())
        ws = 0
        if train:
            for name, level, c in self._GRAD:
                b[name] = bf(level, c)
            ws = max(_lib.lib().vdvc_cnn_wgrad_workspace_bytes(l["cout"], l["cin"]) for l in LAYERS)
        b["ws"] = torch.empty(max(ws, 1 << 16), dtype=torch.uint8, device=D.device())
        b["loss"] = torch.zeros(1, dtype=torch.float64, device=D.device())
        return b

    # ---- forward / backward --------------------------------------------------------

    def _conv(self, name, src, scs, scoff, out, ocs, ocoff, geom, out_f32=False):
        l = LAYER[name]
        _, bptr = self._wptr(name)
        _lib.check(_lib.lib().vdvc_cnn_conv(src.data_ptr(), scs, scoff, l["cin"], self.wf[name].data_ptr(), bptr,
                                            l["cout"], int(l["relu"]), out.data_ptr(), int(out_f32), ocs, ocoff, 0,
                                            C.byref(geom), D.stream()), f"conv {name}")

    def _up(self, src, scs, scoff, m, dst, dcs, dcoff, n, nch):
        _lib.check(_lib.lib().vdvc_cnn_upsample2(src.data_ptr(), scs, scoff, *m, dst.data_ptr(), dcs, dcoff, *n, nch,
                                                 D.stream()), "upsample2")

    def forward(self, G, train=True, slot=0):
        """Run the network on buffers(G)['x']; returns the FP32 output
        (npos(G1) x 8, channels [0,3) used)."""
        b = self.buffers(G, train, slot)
        g0, g1, g2, g3 = b["lv"]
        self._conv("e1", b["x"], 2, 0, b["e1"], 32, 0, fwd_geom(g0, g0, 1))
        self._conv("e2a", b["e1"], 32, 0, b["e2a"], 64, 0, fwd_geom(g1, g0, 2))
        self._conv("e2b", b["e2a"], 64, 0, b["cat2"], 128, 64, fwd_geom(g1, g1, 1))
        self._conv("e3a", b["cat2"], 128, 64, b["e3a"], 128, 0, fwd_geom(g2, g1, 2))
        self._conv("e3b", b["e3a"], 128, 0, b["cat3"], 256, 128, fwd_geom(g2, g2, 1))
        self._conv("e4a", b["cat3"], 256, 128, b["e4a"], 128, 0, fwd_geom(g3, g2, 2))
        self._conv("e4b", b["e4a"], 128, 0, b["e4b"], 128, 0, fwd_geom(g3, g3, 1))
        self._up(b["e4b"], 128, 0, g3, b["cat3"], 256, 0, g2, 128)
        self._conv("d3", b["cat3"], 256, 0, b["d3"], 64, 0, fwd_geom(g2, g2, 1))
        self._up(b["d3"], 64, 0, g2, b["cat2"], 128, 0, g1, 64)
        self._conv("d2", b["cat2"], 128, 0, b["d2"], 32, 0, fwd_geom(g1, g1, 1))
        self._conv("out", b["d2"], 32, 0, b["pred"], 8, 0, fwd_geom(g1, g1, 1), out_f32=True)
        return b["pred"]

    def loss(self, G, target, want_grad=True, scale=1.0):
        """MSE of the output against target (FP32 CUDA (npos(G1), 3)); with
        want_grad the output gradient goes to the dp buffer.  Returns the
        device loss scalar (float64 tensor of 1)."""
        b = self.buffers(G, want_grad)
        npos = _npos(b["lv"][1])
        _lib.check(_lib.lib().vdvc_cnn_mse(b["pred"].data_ptr(), 8, target.data_ptr(), npos, b["loss"].data_ptr(),
                                           b["dp"].data_ptr() if want_grad else None, 16, float(scale),
                                           b["ws"].data_ptr(), b["ws"].numel(), D.stream()), "cnn_mse")
        return b["loss"]

    def _back(self, name, dy, dcs, dcoff, x, xcs, xcoff, geom_fwd, b, accumulate):
        l = LAYER[name]
        L = _lib.lib()
        wptr, bptr = self._wptr(name, grad=True)
        ws = b["ws"]
        _lib.check(L.vdvc_cnn_conv_wgrad(dy.data_ptr(), dcs, dcoff, l["cout"], x.data_ptr(), xcs, xcoff, l["cin"],
                                         C.byref(geom_fwd), wptr, int(accumulate), ws.data_ptr(), ws.numel(),
                                         D.stream()), f"wgrad {name}")
        npos = geom_fwd.nx * geom_fwd.ny * geom_fwd.nz
        _lib.check(L.vdvc_cnn_bias_grad(dy.data_ptr(), dcs, dcoff, l["cout"], npos, bptr, int(accumulate),
                                        ws.data_ptr(), ws.numel(), D.stream()), f"bias_grad {name}")

    def _dconv(self, name, dy, dcs, dcoff, out, ocs, ocoff, out_grid, src_grid, accumulate=False):
        """Input gradient of layer `name` (its transposed weights, adjoint
        geometry), written (or added, accumulate) to out."""
        l = LAYER[name]
        geom = bwd_geom(out_grid, src_grid, l["stride"])
        _lib.check(_lib.lib().vdvc_cnn_conv(dy.data_ptr(), dcs, dcoff, _pad(l["cout"], 16), self.wb[name].data_ptr(),
                                            None, l["cin"], 0, out.data_ptr(), 0, ocs, ocoff, int(accumulate),
                                            C.byref(geom), D.stream()), f"input grad {name}")

    def _relu_bwd(self, d, a):
        _lib.check(_lib.lib().vdvc_cnn_relu_bwd(d.data_ptr(), a.data_ptr(), d.numel(), D.stream()), "relu_bwd")

    def _up_bwd(self, dfine, fcs, fcoff, n, dcoarse, ccs, ccoff, m, nch):
        _lib.check(_lib.lib().vdvc_cnn_upsample2_bwd(dfine.data_ptr(), fcs, fcoff, *n, dcoarse.data_ptr(), ccs, ccoff,
                                                     *m, nch, D.stream()), "upsample2_bwd")

    def backward(self, G, accumulate=False):
        """Parameter gradients (into self.grad; added when accumulate) from
        the output gradient in the dp buffer.  Where a skip connection's two
        gradients meet, the second input gradient is added onto the first
        in the concatenation's gradient buffer; a ReLU mask applied to a
        whole concatenation touches only channels already consumed."""
        b = self.buffers(G)
        g0, g1, g2, g3 = b["lv"]
        acc = accumulate
        self._back("out", b["dp"], 16, 0, b["d2"], 32, 0, fwd_geom(g1, g1, 1), b, acc)
        self._dconv("out", b["dp"], 16, 0, b["dd2"], 32, 0, g1, g1)
        self._relu_bwd(b["dd2"], b["d2"])
        self._back("d2", b["dd2"], 32, 0, b["cat2"], 128, 0, fwd_geom(g1, g1, 1), b, acc)
        self._dconv("d2", b["dd2"], 32, 0, b["dcat2"], 128, 0, g1, g1)
        self._up_bwd(b["dcat2"], 128, 0, g1, b["dd3"], 64, 0, g2, 64)
        self._relu_bwd(b["dd3"], b["d3"])
        self._back("d3", b["dd3"], 64, 0, b["cat3"], 256, 0, fwd_geom(g2, g2, 1), b, acc)
        self._dconv("d3", b["dd3"], 64, 0, b["dcat3"], 256, 0, g2, g2)
        self._up_bwd(b["dcat3"], 256, 0, g2, b["de4b"], 128, 0, g3, 128)
        self._relu_bwd(b["de4b"], b["e4b"])
        self._back("e4b", b["de4b"], 128, 0, b["e4a"], 128, 0, fwd_geom(g3, g3, 1), b, acc)
        self._dconv("e4b", b["de4b"], 128, 0, b["de4a"], 128, 0, g3, g3)
        self._relu_bwd(b["de4a"], b["e4a"])
        self._back("e4a", b["de4a"], 128, 0, b["cat3"], 256, 128, fwd_geom(g3, g2, 2), b, acc)
        # e3b feeds e4a and the concatenation
        self._dconv("e4a", b["de4a"], 128, 0, b["dcat3"], 256, 128, g2, g3, accumulate=True)
        self._relu_bwd(b["dcat3"], b["cat3"])
        self._back("e3b", b["dcat3"], 256, 128, b["e3a"], 128, 0, fwd_geom(g2, g2, 1), b, acc)
        self._dconv("e3b", b["dcat3"], 256, 128, b["de3a"], 128, 0, g2, g2)
        self._relu_bwd(b["de3a"], b["e3a"])
        self._back("e3a", b["de3a"], 128, 0, b["cat2"], 128, 64, fwd_geom(g2, g1, 2), b, acc)
        # e2b feeds e3a and the concatenation
        self._dconv("e3a", b["de3a"], 128, 0, b["dcat2"], 128, 64, g1, g2, accumulate=True)
        self._relu_bwd(b["dcat2"], b["cat2"])
        self._back("e2b", b["dcat2"], 128, 64, b["e2a"], 64, 0, fwd_geom(g1, g1, 1), b, acc)
        self._dconv("e2b", b["dcat2"], 128, 64, b["de2a"], 64, 0, g1, g1)
        self._relu_bwd(b["de2a"], b["e2a"])
        self._back("e2a", b["de2a"], 64, 0, b["e1"], 32, 0, fwd_geom(g1, g0, 2), b, acc)
        self._dconv("e2a", b["de2a"], 64, 0, b["de1"], 32, 0, g0, g1)
        self._relu_bwd(b["de1"], b["e1"])
        self._back("e1", b["de1"], 32, 0, b["x"], 2, 0, fwd_geom(g0, g0, 1), b, acc)

    def adam(self, lr, beta1=0.9, beta2=0.999, eps=1e-8):
        self.step_count += 1
        _lib.check(_lib.lib().vdvc_cnn_adam(self.theta.data_ptr(), self.grad.data_ptr(), self.m.data_ptr(),
                                            self.v.data_ptr(), self.nparam, float(lr), beta1, beta2, eps,
                                            self.step_count, D.stream()), "cnn_adam")
        self.pack()

    # ---- inputs ------------------------------------------------------------------

    def set_input(self, f_vox, g_vox, shape, train=True, flip=0, slot=0, mean_std=None, sums=None):
        """Pool f and g (FP32 vox-layout CUDA tensors of `shape` voxels),
        mirrored along the axes of `flip` (bit 0 x, 1 y, 2 z), into the input
        buffer; returns the input grid.  The standardising statistics come
        from `mean_std` (host [mean_f, std_f, mean_g, std_g]), or from
        `sums` (device, input_moments) without a host read-back, or are
        computed here."""
        G = input_grid(shape)
        b = self.buffers(G, train, slot)
        if sums is not None:
            _lib.check(_lib.lib().vdvc_cnn_pool_input_dev(f_vox.data_ptr(), g_vox.data_ptr(), *shape,
                                                          sums.data_ptr(), int(flip), b["x"].data_ptr(), D.stream()),
                       "cnn_pool_input_dev")
            return G
        ms = mean_std if mean_std is not None else np.array(_mean_std_many(f_vox, g_vox), np.float64)
        _lib.check(_lib.lib().vdvc_cnn_pool_input_mirrored(f_vox.data_ptr(), g_vox.data_ptr(), *shape,
                                                           ms.ctypes.data_as(_lib.pd), int(flip), b["x"].data_ptr(),
                                                           D.stream()), "cnn_pool_input")
        return G

    # mirror sets of the test-time average: the pair itself, then mirrored
    # along x, y and both (the network is not equivariant to mirroring, so
    # the passes' errors are partly independent)
    MIRRORS = {1: (0,), 2: (0, 1), 4: (0, 1, 2, 3)}

    def mirrors_for(self, shape, h, Nx, Ny, Nz, passes):
        """The mirror masks usable for this volume and mesh (a mirrored
        axis needs the pooled and output grids and the mesh to be symmetric
        under the mirror)."""
        ok = [(s - 1) % OUT_STRIDE == 0 and N * h == s - 1 for s, N in zip(shape, (Nx, Ny, Nz))]
        return tuple(m for m in self.MIRRORS[passes] if all(ok[k] or not (m >> k) & 1 for k in range(3)))

    def predict_nodes(self, f_vox, g_vox, shape, h, Nx, Ny, Nz, passes=1, wait=True):
        """Seed U (float64 CUDA tensor, 3 (Nx+1)(Ny+1)(Nz+1)) for a mesh of
        edge h over a volume of `shape` voxels.  passes > 1: the mean of the
        predictions for the pair and its mirror images (1, 2 or 4 passes).

        Everything runs on side streams, ordered after the work already on
        the caller's stream: the image moments and the pooled input of the
        first pass (no host read-back), the mirrored passes' inputs as
        mirror images of that pooled grid (mirrors_for only admits axes
        along which the pooling grid is symmetric; the same windows summed
        in the mirrored FP32 order), the passes concurrently,
        then the nodal resampling.  wait=True: the caller's stream waits for
        the seed and U is returned; wait=False: (U, event) is returned and
        the caller's stream is free for independent work until it waits on
        the event."""
        torch = D.torch()
        L = _lib.lib()
        mirrors = self.mirrors_for(shape, h, Nx, Ny, Nz, passes)
        main = torch.cuda.current_stream()
        U = D.empty(3 * (Nx + 1) * (Ny + 1) * (Nz + 1), np.float64)
        ready = torch.cuda.Event()
        ready.record(main)
        s0 = self._side_stream(0)
        with torch.cuda.stream(s0):
            s0.wait_event(ready)
            sums = D.zeros(4, np.float64)
            ws = D.scratch.get(1 << 16)
            _lib.check(L.vdvc_cnn_input_moments(f_vox.data_ptr(), g_vox.data_ptr(), f_vox.numel(), sums.data_ptr(),
                                                ws.data_ptr(), ws.numel(), D.stream()), "cnn_input_moments")
            G = self.set_input(f_vox, g_vox, shape, train=False, flip=mirrors[0], slot=0, sums=sums)
            pooled = torch.cuda.Event()
            pooled.record(s0)
            preds = [(self.forward(G, train=False, slot=0), mirrors[0], s0)]
        x0 = self.buffers(G, False, 0)["x"]
        for k, flip in enumerate(mirrors[1:], 1):
            st = self._side_stream(k)
            with torch.cuda.stream(st):
                st.wait_event(pooled)
                _lib.check(L.vdvc_cnn_mirror_input(x0.data_ptr(), *G, int(flip ^ mirrors[0]),
                                                   self.buffers(G, False, k)["x"].data_ptr(), D.stream()),
                           "cnn_mirror_input")
                preds.append((self.forward(G, train=False, slot=k), flip, st))
        n = self.buffers(G, train=False)["lv"][1]
        w = 1.0 / len(mirrors)
        with torch.cuda.stream(s0):
            for _, _, st in preds[1:]:
                s0.wait_stream(st)
            for k, (pred, flip, _) in enumerate(preds):
                _lib.check(L.vdvc_cnn_seed_nodes_acc(pred.data_ptr(), 8, *n, h, Nx, Ny, Nz, int(flip), w, int(k > 0),
                                                     U.data_ptr(), D.stream()), "cnn_seed_nodes")
            done = torch.cuda.Event()
            done.record(s0)
        U.record_stream(s0)
        if not wait:
            return U, done
        main.wait_event(done)
        return U

    def _side_stream(self, k):
        streams = self.__dict__.setdefault("_streams", {})
        key = (D.torch().cuda.current_device(), k)
        if key not in streams:
            streams[key] = D.torch().cuda.Stream()
        return streams[key]


def _to_bf16_bits(a):
    """Nearest BF16 (ties to even) of float32 a, as uint16 bit patterns."""
    b = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) >> 16
    return b.astype(np.uint16)


def _from_bf16_bits(b):
    return (np.asarray(b, np.uint32) << 16).view(np.float32)


def _mean_std(x):
    """(mean, population std) of a float32 CUDA tensor, float64 sums on the
    device (vdvc_dot)."""
    return tuple(_mean_std_many(x))


def _mean_std_many(*xs):
    """[mean, std, mean, std, ...] of float32 CUDA tensors: the float64
    sums of every tensor reduced into one device buffer, read back once."""
    L = _lib.lib()
    ws = D.scratch.get(1 << 16)
    sums = D.zeros(2 * len(xs), np.float64)
    for k, x in enumerate(xs):
        n = x.numel()
        _lib.check(L.vdvc_dot_device(x.data_ptr(), None, _lib.F32, n, sums[2 * k:2 * k + 1].data_ptr(),
                                     ws.data_ptr(), ws.numel(), D.stream()), "dot")
        _lib.check(L.vdvc_dot_device(x.data_ptr(), x.data_ptr(), _lib.F32, n, sums[2 * k + 1:2 * k + 2].data_ptr(),
                                     ws.data_ptr(), ws.numel(), D.stream()), "dot")
    h = sums.cpu().numpy()
    out = []
    for k, x in enumerate(xs):
        n = x.numel()
        mean = h[2 * k] / n
        var = max(h[2 * k + 1] / n - mean * mean, 0.0)
        out += [float(mean), float(np.sqrt(var)) if var > 0 else 1.0]
    return out
