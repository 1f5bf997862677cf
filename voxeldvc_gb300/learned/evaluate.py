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
and reports the nodal RMS differences between them, each solve's RMS error
against the true field over the recoverable nodes (at least 4 elements
inside the mesh border, with a true deformed position at least one element
inside the volume: elsewhere the deformed position leaves g or its support
is truncated), the fallback rate and the solve times.  Where the plain
pyramid itself lands in a wrong minimum (large rotations), the FP64 solve
does too, and the learned solve is measured against the true field.

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


def _recoverable(n, U_true, size):
    """Boolean mask of the nodes of an n^3 node grid (stride H) that are at
    least 4 elements inside the border and whose true deformed position stays
    at least one element inside the volume."""
    torch = D.torch()
    i = torch.arange(n, device=U_true.device)
    z, y, x = torch.meshgrid(i, i, i, indexing="ij")
    X = torch.stack([x, y, z], -1).reshape(-1, 3).double() * H
    inner = ((X >= 4 * H) & (X <= (n - 1 - 4) * H)).all(1)
    Y = X + U_true.view(-1, 3).double()
    inside = ((Y >= H) & (Y <= size - 1 - H)).all(1)
    return inner & inside


def _rms_on(a, b, mask):
    T = D.torch()
    d = (a.double() - b.double()).view(-1, 3)[mask]
    return float(T.sqrt(T.mean(d ** 2)).item()) if d.numel() else float("nan")


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
        rec = _recoverable(Nx + 1, U_true, maker.size)
        rows.append(dict(seed=seed, seed_rms=_rms(seed_U, U_true), learned_vs_f64=_rms(Ul, U64),
                         learned_vs_plain=_rms(Ul, Up), plain_vs_f64=_rms(Up, U64), plain_vs_true=_rms(Up, U_true),
                         seed_vs_true_rec=_rms_on(seed_U, U_true, rec), learned_vs_true_rec=_rms_on(Ul, U_true, rec),
                         plain_vs_true_rec=_rms_on(Up, U_true, rec), f64_vs_true_rec=_rms_on(U64, U_true, rec),
                         recoverable_frac=float(rec.double().mean().item()),
                         fallback=last.get("seed") != "learned", norm_res=last.get("norm_res"),
                         gn_finest=gn[-1] if gn else -1, t_learned=tl, t_plain=tp, t_f64=t64))
        if (i + 1) % 10 == 0 or i == pairs - 1:
            r = rows[-1]
            log(f"{i + 1:4d}/{pairs}  seed {r['seed_rms']:.3f}  learned-f64 {r['learned_vs_f64']:.4f}  "
                f"plain-f64 {r['plain_vs_f64']:.4f}  learned-true {r['learned_vs_true_rec']:.4f}  "
                f"plain-true {r['plain_vs_true_rec']:.4f}  fallback {r['fallback']}  {tl:.3f} / {tp:.3f} s",
                flush=True)

    def stat(key):
        v = np.array([r[key] for r in rows], np.float64)
        return {"mean": float(v.mean()), "median": float(np.median(v)), "p95": float(np.percentile(v, 95)),
                "max": float(v.max())}

    plain_ok = np.array([r["plain_vs_true_rec"] < 0.1 for r in rows])
    ok_rows = [r for r, k in zip(rows, plain_ok) if k]

    def stat_on(key, sel):
        v = np.array([r[key] for r in sel], np.float64)
        return {"mean": float(v.mean()), "median": float(np.median(v)), "p95": float(np.percentile(v, 95)),
                "max": float(v.max())} if v.size else None

    summary = {"pairs": pairs, "h": H, "size": maker.size,
               "recoverable_node_frac": stat("recoverable_frac"),
               "seed_vs_true_recoverable_rms_vx": stat("seed_vs_true_rec"),
               "learned_vs_true_recoverable_rms_vx": stat("learned_vs_true_rec"),
               "plain_vs_true_recoverable_rms_vx": stat("plain_vs_true_rec"),
               "f64_vs_true_recoverable_rms_vx": stat("f64_vs_true_rec"),
               "plain_correct_rate": float(plain_ok.mean()),
               "learned_correct_rate": float(np.mean([r["learned_vs_true_rec"] < 0.1 for r in rows])),
               "learned_vs_f64_rms_vx_where_plain_correct": stat_on("learned_vs_f64", ok_rows),
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
