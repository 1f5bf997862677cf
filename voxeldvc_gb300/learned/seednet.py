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
            if name != "c1":
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
        p = self.params_numpy()
        arrays = {f"{k}_W": v[0] for k, v in p.items()}
        arrays.update({f"{k}_b": v[1] for k, v in p.items()})
        arrays.update({f"meta_{k}": np.asarray(v) for k, v in meta.items()})
        np.savez(path, **arrays)

    @classmethod
    def load(cls, path=WEIGHTS_PATH):
        z = np.load(path)
        params = {l["name"]: (z[f"{l['name']}_W"], z[f"{l['name']}_b"]) for l in LAYERS}
        net = cls(params)
        net.meta = {k[5:]: z[k] for k in z.files if k.startswith("meta_")}
        return net

    # ---- buffers -----------------------------------------------------------------

    def buffers(self, G):
        """Activation and gradient buffers for input grid G (cached)."""
        G = tuple(int(v) for v in G)
        if G in self._bufs:
            return self._bufs[G]
        torch = D.torch()
        _, n, m = grids(G)
        bf = lambda grid, c: torch.zeros(_npos(grid) * c, dtype=torch.bfloat16, device=D.device())
        b = dict(G=G, n=n, m=m,
                 x=bf(G, 2), a1=bf(G, 16), a2=bf(n, 32), cat=bf(n, 64), a4=bf(m, 32), a5=bf(m, 32), a6=bf(m, 32),
                 a7=bf(n, 16), pred=torch.zeros(_npos(n) * 8, dtype=torch.float32, device=D.device()),
                 d8=bf(n, 16), d7=bf(n, 16), dcat=bf(n, 64), d6=bf(m, 32), d5=bf(m, 32), d4=bf(m, 32),
                 d2=bf(n, 32), d1=bf(G, 16))
        ws = max(_lib.lib().vdvc_cnn_wgrad_workspace_bytes(l["cout"], l["cin"]) for l in LAYERS)
        b["ws"] = torch.empty(max(ws, 1 << 16), dtype=torch.uint8, device=D.device())
        b["loss"] = torch.zeros(1, dtype=torch.float64, device=D.device())
        self._bufs[G] = b
        return b

    # ---- forward / backward --------------------------------------------------------

    def _conv(self, name, src, scs, scoff, cin, out, ocs, ocoff, geom, out_f32=False, relu=None):
        l = LAYER[name]
        _, bptr = self._wptr(name)
        _lib.check(_lib.lib().vdvc_cnn_conv(src.data_ptr(), scs, scoff, cin, self.wf[name].data_ptr(), bptr,
                                            l["cout"], int(l["relu"] if relu is None else relu), out.data_ptr(),
                                            int(out_f32), ocs, ocoff, 0, C.byref(geom), D.stream()), f"conv {name}")

    def forward(self, G):
        """Run the network on buffers(G)['x']; returns the FP32 output
        (npos(n) x 8, channels [0,3) used)."""
        b = self.buffers(G)
        L = _lib.lib()
        G, n, m = b["G"], b["n"], b["m"]
        self._conv("c1", b["x"], 2, 0, 2, b["a1"], 16, 0, fwd_geom(G, G, 1))
        self._conv("c2", b["a1"], 16, 0, 16, b["a2"], 32, 0, fwd_geom(n, G, 2))
        self._conv("c3", b["a2"], 32, 0, 32, b["cat"], 64, 32, fwd_geom(n, n, 1))
        self._conv("c4", b["cat"], 64, 32, 32, b["a4"], 32, 0, fwd_geom(m, n, 2))
        self._conv("c5", b["a4"], 32, 0, 32, b["a5"], 32, 0, fwd_geom(m, m, 1))
        self._conv("c6", b["a5"], 32, 0, 32, b["a6"], 32, 0, fwd_geom(m, m, 1))
        _lib.check(L.vdvc_cnn_upsample2(b["a6"].data_ptr(), 32, 0, *m, b["cat"].data_ptr(), 64, 0, *n, 32,
                                        D.stream()), "upsample2")
        self._conv("c7", b["cat"], 64, 0, 64, b["a7"], 16, 0, fwd_geom(n, n, 1))
        self._conv("c8", b["a7"], 16, 0, 16, b["pred"], 8, 0, fwd_geom(n, n, 1), out_f32=True)
        return b["pred"]

    def loss(self, G, target, want_grad=True, scale=1.0):
        """MSE of the output against target (FP32 CUDA (npos(n), 3)); with
        want_grad the output gradient goes to the d8 buffer.  Returns the
        device loss scalar (float64 tensor of 1)."""
        b = self.buffers(G)
        npos = _npos(b["n"])
        _lib.check(_lib.lib().vdvc_cnn_mse(b["pred"].data_ptr(), 8, target.data_ptr(), npos, b["loss"].data_ptr(),
                                           b["d8"].data_ptr() if want_grad else None, 16, float(scale),
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

    def backward(self, G, accumulate=False):
        """Parameter gradients (into self.grad; added when accumulate) from
        the output gradient in the d8 buffer."""
        b = self.buffers(G)
        L = _lib.lib()
        G, n, m = b["G"], b["n"], b["m"]
        acc = accumulate
        self._back("c8", b["d8"], 16, 0, b["a7"], 16, 0, fwd_geom(n, n, 1), b, acc)
        self._dconv("c8", b["d8"], 16, 0, b["d7"], 16, 0, n, n)
        self._relu_bwd(b["d7"], b["a7"])
        self._back("c7", b["d7"], 16, 0, b["cat"], 64, 0, fwd_geom(n, n, 1), b, acc)
        self._dconv("c7", b["d7"], 16, 0, b["dcat"], 64, 0, n, n)
        _lib.check(L.vdvc_cnn_upsample2_bwd(b["dcat"].data_ptr(), 64, 0, *n, b["d6"].data_ptr(), 32, 0, *m, 32,
                                            D.stream()), "upsample2_bwd")
        self._relu_bwd(b["d6"], b["a6"])
        self._back("c6", b["d6"], 32, 0, b["a5"], 32, 0, fwd_geom(m, m, 1), b, acc)
        self._dconv("c6", b["d6"], 32, 0, b["d5"], 32, 0, m, m)
        self._relu_bwd(b["d5"], b["a5"])
        self._back("c5", b["d5"], 32, 0, b["a4"], 32, 0, fwd_geom(m, m, 1), b, acc)
        self._dconv("c5", b["d5"], 32, 0, b["d4"], 32, 0, m, m)
        self._relu_bwd(b["d4"], b["a4"])
        self._back("c4", b["d4"], 32, 0, b["cat"], 64, 32, fwd_geom(m, n, 2), b, acc)
        # c3 feeds c4 and the concatenation: add c4's input gradient onto
        # the concatenation gradient's c3 channels
        self._dconv("c4", b["d4"], 32, 0, b["dcat"], 64, 32, n, m, accumulate=True)
        # ReLU mask of the whole concatenation: channels [0, 32) are spent
        self._relu_bwd(b["dcat"], b["cat"])
        self._back("c3", b["dcat"], 64, 32, b["a2"], 32, 0, fwd_geom(n, n, 1), b, acc)
        self._dconv("c3", b["dcat"], 64, 32, b["d2"], 32, 0, n, n)
        self._relu_bwd(b["d2"], b["a2"])
        self._back("c2", b["d2"], 32, 0, b["a1"], 16, 0, fwd_geom(n, G, 2), b, acc)
        self._dconv("c2", b["d2"], 32, 0, b["d1"], 16, 0, G, n)
        self._relu_bwd(b["d1"], b["a1"])
        self._back("c1", b["d1"], 16, 0, b["x"], 2, 0, fwd_geom(G, G, 1), b, acc)

    def adam(self, lr, beta1=0.9, beta2=0.999, eps=1e-8):
        self.step_count += 1
        _lib.check(_lib.lib().vdvc_cnn_adam(self.theta.data_ptr(), self.grad.data_ptr(), self.m.data_ptr(),
                                            self.v.data_ptr(), self.nparam, float(lr), beta1, beta2, eps,
                                            self.step_count, D.stream()), "cnn_adam")
        self.pack()

    # ---- inputs ------------------------------------------------------------------

    def set_input(self, f_vox, g_vox, shape):
        """Pool f and g (FP32 vox-layout CUDA tensors of `shape` voxels) into
        the input buffer; returns the input grid."""
        G = input_grid(shape)
        b = self.buffers(G)
        ms = np.array([*_mean_std(f_vox), *_mean_std(g_vox)], np.float64)
        _lib.check(_lib.lib().vdvc_cnn_pool_input(f_vox.data_ptr(), g_vox.data_ptr(), *shape,
                                                  ms.ctypes.data_as(_lib.pd), b["x"].data_ptr(), D.stream()),
                   "cnn_pool_input")
        return G

    def predict_nodes(self, f_vox, g_vox, shape, h, Nx, Ny, Nz):
        """Seed U (float64 CUDA tensor, 3 (Nx+1)(Ny+1)(Nz+1)) for a mesh of
        edge h over a volume of `shape` voxels."""
        G = self.set_input(f_vox, g_vox, shape)
        pred = self.forward(G)
        n = self.buffers(G)["n"]
        U = D.empty(3 * (Nx + 1) * (Ny + 1) * (Nz + 1), np.float64)
        _lib.check(_lib.lib().vdvc_cnn_seed_nodes(pred.data_ptr(), 8, *n, h, Nx, Ny, Nz, U.data_ptr(), D.stream()),
                   "cnn_seed_nodes")
        return U


def _mean_std(x):
    """(mean, population std) of a float32 CUDA tensor, float64 sums on the
    device (vdvc_dot)."""
    L = _lib.lib()
    ws = D.scratch.get(1 << 16)
    s = C.c_double(0.0)
    ss = C.c_double(0.0)
    n = x.numel()
    _lib.check(L.vdvc_dot(x.data_ptr(), None, _lib.F32, n, C.byref(s), ws.data_ptr(), ws.numel(), D.stream()), "dot")
    _lib.check(L.vdvc_dot(x.data_ptr(), x.data_ptr(), _lib.F32, n, C.byref(ss), ws.data_ptr(), ws.numel(),
                          D.stream()), "dot")
    mean = s.value / n
    var = max(ss.value / n - mean * mean, 0.0)
    return mean, float(np.sqrt(var)) if var > 0 else 1.0
