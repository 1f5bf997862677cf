"""Batched solves (engine/batch.py): every problem of a series with uneven
ROIs and element sizes gives exactly its own multiscale solve, with the
default schedule and with the autotuner's."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def series(cuda):
    import torch
    from voxeldvc_gb300 import synth
    shape = (97, 97, 97)
    f = synth.texture(shape, 60, seed=5, cyl_seed=6)
    gs = []
    for k in range(3):
        ez = 0.004 * (k + 1)
        params = [0.3 * k, -0.2, 0.1, *np.diag([-0.4 * ez, -0.4 * ez, ez]).reshape(-1), 48.0, 48.0, 48.0]
        gs.append(synth.vox_to_pix(synth.warp(f, shape, synth.FIELD_AFFINE, params, 0.01, seed=20 + k), shape))
    f_pix = synth.vox_to_pix(f, shape)
    problems = [dict(origin=(3, 5, 2), h=8, mesh=(8, 8, 9)),
                dict(origin=(20, 10, 30), h=4, mesh=(12, 10, 14)),
                dict(origin=(0, 8, 4), h=16, mesh=(4, 5, 4))]
    return torch, f_pix, gs, problems


def _solo(torch, f_pix, g_pix, p, kw):
    from voxeldvc_gb300.engine import correlate_gpu as CG
    h = p["h"]
    (x0, y0, z0), (Nx, Ny, Nz) = p["origin"], p["mesh"]
    sl = (slice(x0, x0 + Nx * h + 1), slice(y0, y0 + Ny * h + 1), slice(z0, z0 + Nz * h + 1))
    return CG.multiscale_correlate_gpu(f_pix[sl], g_pix[sl], Nx, Ny, Nz, h, xp=np, l0=4.5 * h, **kw)


KW = dict(scales=(1, 0), fft_prealign=True, dynamic_mask=True, freeze_mask_after=4, maxiter=20, eps=1e-3,
          pcg_tol=1e-6, pcg_max_iter=2000, glt=0.0)


def test_batch_matches_individual_solves(series, tmp_path, monkeypatch):
    torch, f_pix, gs, problems = series
    from voxeldvc_gb300.engine import batch as B, geometry_dvc as G
    Kl = G.build_K_ref_laplacian()
    stats = []
    out = B.batch_multiscale_correlate_gpu(f_pix, gs, problems, np, l0_factor=4.5, K_ref_laplacian=Kl,
                                           stats=stats, **KW)
    assert len(out) == 3 and [s["scale"] for s in stats] == [1, 0]
    for i, p in enumerate(problems):
        U1, r1, d1 = _solo(torch, f_pix, gs[i], p, dict(KW, K_ref_laplacian=Kl))
        U, r, d = out[i]
        assert U.shape == U1.shape and r.shape == r1.shape
        assert np.abs(U - U1).max() < 1e-6, i
        assert np.abs(r - r1).max() < 1e-5, i
    # the schedule does not change the arithmetic: serialised streams, chunk 1
    out2 = B.batch_multiscale_correlate_gpu(f_pix, gs, problems, np, l0_factor=4.5, K_ref_laplacian=Kl,
                                            pcg_chunk=1, concurrent=False, **KW)
    for i in range(3):
        assert np.abs(out2[i][0] - out[i][0]).max() < 1e-6
    # the autotuner measures, caches and reuses its choice
    cache = tmp_path / "tune.json"
    monkeypatch.setenv("VDVC_TUNE_CACHE", str(cache))
    st3 = []
    out3 = B.batch_multiscale_correlate_gpu(f_pix, gs, problems, np, l0_factor=4.5, K_ref_laplacian=Kl, tune=True,
                                            stats=st3, **KW)
    assert cache.exists()
    import json
    entries = json.loads(cache.read_text())
    assert len(entries) == 2  # one problem class per level
    for i in range(3):
        assert np.abs(out3[i][0] - out[i][0]).max() < 1e-6
    st4 = []
    B.batch_multiscale_correlate_gpu(f_pix, gs, problems, np, l0_factor=4.5, K_ref_laplacian=Kl, stats=st4, **KW)
    assert [s["schedule"] for s in st4] == [s["schedule"] for s in st3]


def test_batch_rejects_bad_problems(series):
    torch, f_pix, gs, problems = series
    from voxeldvc_gb300.engine import batch as B
    with pytest.raises(ValueError):
        B.batch_multiscale_correlate_gpu(f_pix, gs[:2], problems, np)
    bad = [dict(origin=(60, 0, 0), h=8, mesh=(8, 8, 8))]
    with pytest.raises(ValueError):
        B.batch_multiscale_correlate_gpu(f_pix, gs[:1], bad, np)
    odd = [dict(origin=(0, 0, 0), h=6, mesh=(4, 4, 4))]
    with pytest.raises(ValueError):
        B.batch_multiscale_correlate_gpu(f_pix, gs[:1], odd, np, scales=(2, 1, 0))
