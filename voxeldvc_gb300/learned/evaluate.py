"""Accuracy of the learned initial guess on held-out pairs.

Each held-out seed (below HELD_OUT_LIMIT, disjoint from the training seeds)
gives a 513^3 pair of the training family (affine + 16^3 cubic B-spline
field, see train.py).  On it this runs, at h = 8 with the `voxeldvc run`
settings (Laplacian l0 = 4.5 h, dynamic mask frozen after 4 iterations,
eps 1e-3, PCG tol 1e-6):
  * the learned seed alone: its RMS error against the true nodal field;
  * the learned seed + precision-form solve (learned_correlate_gpu), with
    its fallback to the plain multiscale solve;
  * the plain FP32 multiscale solve (scales 2, 1, 0, FFT seed);
  * the same solve in FP64 on the GPU -- the FP64 reference at this size;
and reports the nodal RMS differences between them, the fallback rate and
the median solve times.

    python -m voxeldvc_gb300.learned.evaluate --pairs 200 --out eval.json
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from .. import _device as D
from ..engine import correlate_gpu as CG, geometry_dvc as G
from . import solve as LS
from .train import PairMaker, HELD_OUT_LIMIT

H = 8


def _pix(vox, shape):
    nx, ny, nz = shape
    return vox.view(nz, ny, nx).permute(2, 1, 0).contiguous()


def _rms(a, b):
    T = D.torch()
    return float(T.sqrt(T.mean((a.double() - b.double()) ** 2)).item())


def evaluate(pairs=200, net=None, log=print):
    torch = D.torch()
    maker = PairMaker()
    net = net or LS.default_net()
    Nx = Ny = Nz = (maker.size - 1) // H
    kw = dict(l0=4.5 * H, K_ref_laplacian=G.build_K_ref_laplacian(), dynamic_mask=True, freeze_mask_after=4,
              maxiter=30, eps=1e-3, pcg_tol=1e-6, pcg_max_iter=2000, glt=0.0, disp=False)

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        return out, time.perf_counter() - t0

    rows = []
    for i in range(pairs):
        seed = HELD_OUT_LIMIT - 1000 - i
        f_vox, g_vox, shape, target = maker.make(seed)
        f, g = _pix(f_vox, shape), _pix(g_vox, shape)
        U_true = target.view(-1)
        seed_U = LS.learned_seed(f, g, Nx, Ny, Nz, H, net=net)
        st = []
        (Ul, _, _), tl = timed(lambda: LS.learned_correlate_gpu(f, g, Nx, Ny, Nz, H, torch, net=net,
                                                                precision="mixed", stats=st, **kw))
        (Up, _, _), tp = timed(lambda: CG.multiscale_correlate_gpu(f, g, Nx, Ny, Nz, H, xp=torch, scales=(2, 1, 0),
                                                                   fft_prealign=True, **kw))
        (U64, _, _), t64 = timed(lambda: CG.multiscale_correlate_gpu(f, g, Nx, Ny, Nz, H, xp=torch, scales=(2, 1, 0),
                                                                     fft_prealign=True, dtype=np.float64, **kw))
        last = st[-1] if st else {}
        gn = [s["gn_iters"] for s in st if "gn_iters" in s]
        rows.append(dict(seed=seed, seed_rms=_rms(seed_U, U_true), learned_vs_f64=_rms(Ul, U64),
                         learned_vs_plain=_rms(Ul, Up), plain_vs_f64=_rms(Up, U64), plain_vs_true=_rms(Up, U_true),
                         fallback=last.get("seed") != "learned", norm_res=last.get("norm_res"),
                         gn_finest=gn[-1] if gn else -1, t_learned=tl, t_plain=tp, t_f64=t64))
        if (i + 1) % 10 == 0 or i == pairs - 1:
            r = rows[-1]
            log(f"{i + 1:4d}/{pairs}  seed {r['seed_rms']:.3f}  learned-f64 {r['learned_vs_f64']:.4f}  "
                f"plain-f64 {r['plain_vs_f64']:.4f}  fallback {r['fallback']}  {tl:.3f} / {tp:.3f} s", flush=True)

    def stat(key):
        v = np.array([r[key] for r in rows], np.float64)
        return {"mean": float(v.mean()), "median": float(np.median(v)), "p95": float(np.percentile(v, 95)),
                "max": float(v.max())}

    summary = {"pairs": pairs, "h": H, "size": maker.size,
               "seed_rms_vx": stat("seed_rms"), "learned_vs_f64_rms_vx": stat("learned_vs_f64"),
               "learned_vs_plain_rms_vx": stat("learned_vs_plain"), "plain_vs_f64_rms_vx": stat("plain_vs_f64"),
               "plain_vs_true_rms_vx": stat("plain_vs_true"),
               "fallback_rate": float(np.mean([r["fallback"] for r in rows])),
               "within_0.02_vx_of_f64": float(np.mean([r["learned_vs_f64"] <= 0.02 for r in rows])),
               "t_learned_s": stat("t_learned"), "t_plain_s": stat("t_plain"), "t_f64_s": stat("t_f64"),
               "gn_finest_learned": stat("gn_finest")}
    return summary, rows


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--pairs", type=int, default=200)
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    summary, rows = evaluate(a.pairs)
    print(json.dumps(summary))
    if a.out:
        with open(a.out, "w") as fh:
            json.dump({"summary": summary, "pairs": rows}, fh, indent=1)


if __name__ == "__main__":
    main()
