"""Generate the golden vectors of tests/golden/*.npz by running the
reference's own engine code (voxelDVC, src/voxeldvc/engine/*) on NumPy.

Run it with the reference's `src` directory given explicitly:

    python tests/golden/make_golden.py --reference-src <voxelDVC>/src [case ...]

(or with VOXELDVC_REF_SRC set).  Each .npz stores the seeded inputs (or, for
the benchmark-family solves, the digest of inputs that `oracle/workload_inputs.py`
regenerates from seeds) together with the reference outputs, so the tests
replay the exact same cases on machines without a copy of the reference.
The reference cannot be imported at test time.
"""
from __future__ import annotations

import os
import sys

import numpy as np


def _reference_src():
    for i, a in enumerate(sys.argv[1:], 1):
        if a == "--reference-src" and i + 1 < len(sys.argv):
            path = sys.argv[i + 1]
            del sys.argv[i:i + 2]
            return path
        if a.startswith("--reference-src="):
            del sys.argv[i]
            return a.split("=", 1)[1]
    path = os.environ.get("VOXELDVC_REF_SRC")
    if not path:
        sys.exit("make_golden.py: pass --reference-src <voxelDVC checkout>/src (or set VOXELDVC_REF_SRC)")
    return path


REF_SRC = _reference_src()
if not os.path.isdir(os.path.join(REF_SRC, "voxeldvc")):
    sys.exit(f"make_golden.py: no voxeldvc package under {REF_SRC}")
if REF_SRC not in sys.path:
    sys.path.insert(0, REF_SRC)

from voxeldvc.engine import geometry_dvc as G  # noqa: E402
from voxeldvc.engine import kernels_dvc as KD  # noqa: E402
from voxeldvc.engine import correlate_gpu as CG  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def _texture(shape, rng, sigma=1.5, zero_frac=0.0):
    from scipy.ndimage import gaussian_filter
    t = gaussian_filter(rng.standard_normal(shape), sigma)
    t = (t - t.min()) / (t.max() - t.min()) + 0.05
    if zero_frac > 0:
        t[rng.random(shape) < zero_frac] = 0.0
    return t


def geometry():
    d = {}
    for h in (1, 2, 3, 4, 5, 8):
        N, w = G.build_N_stencil(h)
        d[f"N_h{h}"], d[f"w_h{h}"] = N, w
        for i, a in enumerate(G.VoxelCenterStencil(h)):
            d[f"vcs{i}_h{h}"] = a
    d["K_lap"] = G.build_K_ref_laplacian()
    for nu in (0.0, 0.3, 0.45):
        d[f"K_el_{nu}"] = G.build_K_ref(nu)
    d["shape_grads"] = G._shape_grads(0.2, 0.7, 0.4)
    d["B_matrix"] = G._B_matrix(-0.3, 0.5, 0.9)[0]
    for (Nx, Ny, Nz) in ((3, 2, 2), (1, 1, 1), (2, 4, 3)):
        tag = f"{Nx}_{Ny}_{Nz}"
        ni = G.build_node_index(Nx, Ny, Nz)
        d[f"node_index_{tag}"] = ni
        d[f"interior_{tag}"] = G.build_interior_dof_mask(Nx, Ny, Nz)
        d[f"elem_nodes_{tag}"] = G.element_node_ids(ni, Nx, Ny, Nz)
        e = np.arange(Nx * Ny * Nz, dtype=np.int32)
        d[f"elem_dofs_{tag}"] = KD.get_elem_dofs(e, Nx, Ny, np)
        for h in (1, 3, 4):
            d[f"vox_offsets_{tag}_h{h}"] = KD.get_voxel_offsets(h, Nx, Ny, np)
            d[f"vox_origins_{tag}_h{h}"] = KD.get_elem_voxel_origins(e, h, Nx, Ny, np)
    np.savez_compressed(os.path.join(OUT, "geometry.npz"), **d)


def operators(name, Nx, Ny, Nz, h, seed):
    rng = np.random.default_rng(seed)
    Nvx, Nvy, Nvz = Nx * h + 1, Ny * h + 1, Nz * h + 1
    Nvox = Nvx * Nvy * Nvz
    Ndof = 3 * (Nx + 1) * (Ny + 1) * (Nz + 1)
    N, w = G.build_N_stencil(h)
    K_lap = G.build_K_ref_laplacian()
    K_el = G.build_K_ref(0.3)
    inp = {
        "dims": np.array([Nx, Ny, Nz, h]),
        "grad": rng.standard_normal((Nvox, 3)).astype(np.float32),
        "mask": rng.random(Nvox) < 0.85,
        "v": rng.standard_normal(Ndof).astype(np.float32),
        "res": rng.standard_normal(Nvox).astype(np.float32),
        "U": (1.5 * rng.standard_normal(Ndof)).astype(np.float32),
        "f_pix": _texture((Nvx, Nvy, Nvz), rng, zero_frac=0.05).astype(np.float32),
        "g_pix": _texture((Nvx + 3, max(2, Nvy - 1), Nvz + 2), rng, zero_frac=0.05).astype(np.float32),
        "g_origin": np.array([1, 0, 2]),
        "interior": G.build_interior_dof_mask(Nx, Ny, Nz).astype(np.float32),
    }
    inp["b_pcg"] = rng.standard_normal(Ndof).astype(np.float32)
    out = {}
    out["matvec_H"] = KD.matvec_H(inp["v"], inp["grad"], inp["mask"], N, w, h, Nx, Ny, Nz, np)
    out["matvec_H_f64"] = KD.matvec_H(inp["v"].astype(np.float64), inp["grad"].astype(np.float64), inp["mask"], N,
                                      w, h, Nx, Ny, Nz, np)
    out["diag_H"] = KD.build_diagonal_H(inp["grad"], inp["mask"], N, w, h, Nx, Ny, Nz, Ndof, np)
    out["compute_b"] = CG.compute_b_gpu(inp["res"], inp["mask"], inp["grad"], N, w, h, Nx, Ny, Nz, Ndof, np)
    out["matvec_K_lap"] = KD.matvec_K_ref(inp["v"], K_lap, h, Nx, Ny, Nz, np)
    out["diag_K_lap"] = KD.build_diagonal_K_ref(K_lap, h, Nx, Ny, Nz, Ndof, np)
    out["matvec_eqgap"] = KD.matvec_equilibrium_gap(inp["v"].astype(np.float64), K_el, inp["interior"], h, Nx, Ny,
                                                    Nz, np)
    out["diag_eqgap"] = KD.build_diagonal_equilibrium_gap(K_el, inp["interior"], h, Nx, Ny, Nz, Ndof, np)
    out["stats"] = np.array(CG.masked_quadpoint_mean_std(inp["res"], inp["mask"], h, Nx, Ny, Nz, np))
    out["interp"] = CG.interp_field_vox(inp["U"], N, h, Nx, Ny, Nz, np)
    gv, gm = CG.sample_deformed_field(inp["U"], inp["g_pix"], N, h, Nx, Ny, Nz, np,
                                      g_origin=tuple(int(o) for o in inp["g_origin"]), mask0_vox=inp["mask"])
    out["sample_g"], out["sample_mask"] = gv, gm
    f_vox, grad_f = CG.image_grad_and_values(inp["f_pix"], np, dtype=np.float32)
    out["f_vox"], out["grad_f"] = f_vox, grad_f
    mask0 = f_vox > 0.0
    out["eroded"] = CG.erode_mask0_vox(mask0, Nvx, Nvy, Nvz, np)
    # PCG on (H + ll R) with the Jacobi preconditioner of the solve
    ll = 0.37
    dg = KD.build_diagonal_H(inp["grad"], inp["mask"], N, w, h, Nx, Ny, Nz, Ndof, np) + \
        ll * KD.build_diagonal_K_ref(K_lap, h, Nx, Ny, Nz, Ndof, np)
    Minv = 1.0 / (dg + 1e-5 * float(dg.min()))

    def A(x):
        return KD.matvec_H(x, inp["grad"], inp["mask"], N, w, h, Nx, Ny, Nz, np) + \
            ll * KD.matvec_K_ref(x, K_lap, h, Nx, Ny, Nz, np)

    out["pcg_x"] = KD.pcg(A, inp["b_pcg"], Minv, np, max_iter=300, tol=1e-7)
    out["pcg_ll"] = np.array(ll)
    np.savez_compressed(os.path.join(OUT, f"ops_{name}.npz"), **inp, **{"out_" + k: v for k, v in out.items()})


def _sinusoid_problem():
    # a smooth texture with a rigid 1-voxel shift, 2x2x2 elements of h=8
    from scipy.ndimage import shift
    n = 17
    x = np.arange(n)
    X, Y, Z = np.meshgrid(x, x, x, indexing='ij')
    f = (np.sin(2 * np.pi * X / n) + np.sin(2 * np.pi * Y / n) + np.sin(2 * np.pi * Z / n)
         + 0.5 * np.cos(2 * np.pi * (X + Y) / n))
    g = shift(f, (1.0, 0, 0), order=3, mode='nearest')
    return f, g


def _warped_problem(Nx, Ny, Nz, h, seed, shift=(0.8, -0.6, 0.4), pad=0):
    from scipy.ndimage import map_coordinates
    rng = np.random.default_rng(seed)
    shp = (Nx * h + 1, Ny * h + 1, Nz * h + 1)
    big = tuple(s + 8 for s in shp)
    t = _texture(big, rng, sigma=1.2)
    f = t[4:4 + shp[0], 4:4 + shp[1], 4:4 + shp[2]].copy()
    X = np.indices(shp).astype(np.float64)
    u = [shift[0] + 0.01 * (X[0] - shp[0] / 2), shift[1] - 0.004 * (X[1] - shp[1] / 2),
         shift[2] + 0.006 * (X[2] - shp[2] / 2)]
    coords = np.stack([X[a] - u[a] + 4 for a in range(3)])
    g = map_coordinates(t, coords.reshape(3, -1), order=1, mode='nearest').reshape(shp)
    if pad:
        f[:pad] = 0.0
        g[-pad:] = 0.0
    return f.astype(np.float32), g.astype(np.float32)


def solves():
    K_lap = G.build_K_ref_laplacian()
    K_el = G.build_K_ref(0.3)
    f, g = _sinusoid_problem()
    kw = dict(K_ref_laplacian=K_lap, l0=4.5 * 8, maxiter=20, eps=1e-3, disp=False)
    U, res, dU = CG.correlate_gpu(f, g, 2, 2, 2, 8, xp=np, **kw)
    Um, resm, dUm = CG.multiscale_correlate_gpu(f, g, 2, 2, 2, 8, xp=np, scales=(2, 1, 0),
                                                K_ref_laplacian=K_lap, l0=4.5 * 8, maxiter=30, eps=1e-3,
                                                disp=False)
    np.savez_compressed(os.path.join(OUT, "solve_sinusoid.npz"), f=f, g=g, U=U, res=res, dU=dU, U_ms=Um,
                        res_ms=resm, dU_ms=dUm)

    f2, g2 = _warped_problem(4, 4, 4, 4, seed=5, pad=2)
    kw2 = dict(K_ref_laplacian=K_lap, l0=2 * 4, maxiter=12, eps=1e-4, disp=False, dynamic_mask=True,
               freeze_mask_after=2, glt=0.0)
    U2, res2, dU2 = CG.correlate_gpu(f2, g2, 4, 4, 4, 4, xp=np, **kw2)
    np.savez_compressed(os.path.join(OUT, "solve_dynamic.npz"), f=f2, g=g2, U=U2, res=res2, dU=dU2)

    f3, g3 = _warped_problem(3, 3, 3, 4, seed=6)
    kw3 = dict(K_ref_laplacian=K_lap, K_ref_elastic=K_el, reg_type='equilibrium_gap', reg_exponent=4,
               l0=4.5 * 4, maxiter=10, eps=1e-4, disp=False, dynamic_mask=True, freeze_mask_after=4)
    U3, res3, dU3 = CG.correlate_gpu(f3, g3, 3, 3, 3, 4, xp=np, **kw3)
    np.savez_compressed(os.path.join(OUT, "solve_eqgap.npz"), f=f3, g=g3, U=U3, res=res3, dU=dU3)

    f4, g4 = _warped_problem(4, 3, 2, 8, seed=7, shift=(2.6, -1.2, 0.9))
    U4, res4, dU4 = CG.multiscale_correlate_gpu(f4, g4, 4, 3, 2, 8, xp=np, scales=(2, 1, 0), K_ref_laplacian=K_lap,
                                                l0=4.5 * 8, maxiter=20, eps=1e-3, disp=False, dynamic_mask=True,
                                                freeze_mask_after=4, fft_prealign=True)
    np.savez_compressed(os.path.join(OUT, "solve_multiscale.npz"), f=f4, g=g4, U=U4, res=res4, dU=dU4)


def fft_cases():
    rng = np.random.default_rng(42)
    f = rng.uniform(0, 1, size=(32, 32, 32))
    g = np.roll(f, (3, -2, 1), axis=(0, 1, 2))
    d1 = CG.fft_rigid_shift(f, g, np)
    f2 = rng.uniform(0, 1, size=(20, 24, 18))
    g2 = np.roll(rng.uniform(0, 1, size=(22, 20, 18)), (-4, 5, 2), axis=(0, 1, 2))
    g2[:20, :20, :18] = np.roll(f2[:20, :20, :18], (-4, 5, 2), axis=(0, 1, 2))
    d2 = CG.fft_rigid_shift(f2, g2, np)
    np.savez_compressed(os.path.join(OUT, "fft.npz"), f1=f, g1=g, d1=d1, f2=f2, g2=g2, d2=d2)


def affine_cases():
    """A smooth texture and its image under a known affine, x' = A (x - c) + c
    + t with f(x) ~ g(x'); the reference's prealign / refine results on it and
    its ZNCC cost at a few parameter vectors."""
    from scipy.ndimage import map_coordinates
    rng = np.random.default_rng(9)
    n = 41
    f = (_texture((n, n, n), rng, sigma=1.6) * 100.0).astype(np.float32)
    A = CG._build_affine_matrix(np.array([0.03, -0.02, 0.04, 1.02, 0.98, 1.01]))
    t = np.array([1.5, -2.0, 0.7])
    c = np.full(3, (n - 1) / 2.0)
    Y = np.indices((n, n, n)).reshape(3, -1).astype(np.float64)
    X = np.linalg.solve(A, Y - c[:, None] - t[:, None]) + c[:, None]
    g = map_coordinates(f, X, order=1, mode='constant', cval=0.0).reshape(n, n, n).astype(np.float32)
    costs = []
    ps = [np.array([0, 0, 0, 1, 1, 1, 0, 0, 0.0]), np.array([0.03, -0.02, 0.04, 1.02, 0.98, 1.01, 0.75, -1.0, 0.35]),
          np.array([0.1, 0.05, -0.05, 0.95, 1.05, 1.0, -0.5, 0.5, 1.0])]
    f_d, g_d = f[::2, ::2, ::2], g[::2, ::2, ::2]
    cd = np.array([(s - 1) / 2.0 for s in f_d.shape])
    Xf = np.stack([a.ravel() for a in np.meshgrid(*[np.arange(s) for s in f_d.shape], indexing='ij')]).astype(float)
    for p in ps:
        Xp = CG._build_affine_matrix(p) @ (Xf - cd[:, None]) + cd[:, None] + p[6:9, None]
        inb = np.all([(Xp[a] >= 0) & (Xp[a] <= g_d.shape[a] - 1) for a in range(3)], axis=0)
        costs.append(CG._zncc_masked(f_d.ravel(), CG._map_coordinates(g_d, Xp, np, order=1), inb, np))
    Ap, tp, cp, info = CG.affine_prealign(f, g, np, decimate=2, maxiter=60)
    Ar, tr, rinfo = CG.affine_refine_gn(f, g, np, Ap, tp, cp, sigmas=(2.0, 0.0), max_iter=20)
    np.savez_compressed(os.path.join(OUT, "affine.npz"), f=f, g=g, A_true=A, t_true=t, ps=np.stack(ps),
                        costs=np.array(costs), A_pre=Ap, t_pre=tp, c_pre=cp, cost_final=info['cost_final'],
                        A_ref=Ar, t_ref=tr, rms_initial=rinfo['rms_initial'], rms_final=rinfo['rms_final'],
                        iters=np.array(rinfo['iters']))


def post_cases():
    """Post-solve voxel stages (engine/write_output.py): push_field_forward
    in both orders and modes, on float and label fields, and compute_zncc."""
    from voxeldvc.engine import write_output as W
    rng = np.random.default_rng(31)
    Nx, Ny, Nz, h = 3, 2, 2, 4
    shape = (Nx * h + 1, Ny * h + 1, Nz * h + 1)
    f32 = _texture(shape, rng).astype(np.float32)
    f64 = _texture(shape, rng)
    lab = (rng.random(shape) < 0.4).astype(np.uint8) * 3
    U = rng.standard_normal(3 * (Nx + 1) * (Ny + 1) * (Nz + 1)) * 1.7
    d = dict(f32=f32, f64=f64, lab=lab, U=U, dims=np.array([Nx, Ny, Nz, h]))
    for name, fld in (("f32", f32), ("f64", f64)):
        d[f"{name}_o1_nearest"] = W.push_field_forward(fld, U, Nx, Ny, Nz, h, order=1, mode="nearest")
        d[f"{name}_o1_constant"] = W.push_field_forward(fld, U, Nx, Ny, Nz, h, order=1, mode="constant", cval=-1.0)
        d[f"{name}_o0_constant"] = W.push_field_forward(fld, U, Nx, Ny, Nz, h, order=0, mode="constant", cval=7.0)
    d["lab_o0_nearest"] = W.push_field_forward(lab, U, Nx, Ny, Nz, h, order=0, mode="nearest")
    # integer intensity fields at order 1: the sampler's integer output rounding
    d["u16"] = (f64 * 3000.0).astype(np.uint16)
    d["u16_o1_nearest"] = W.push_field_forward(d["u16"], U, Nx, Ny, Nz, h, order=1, mode="nearest")
    d["lab_o1_nearest"] = W.push_field_forward(lab * 40, U, Nx, Ny, Nz, h, order=1, mode="nearest")
    d["lab_o0_constant"] = W.push_field_forward(lab, U, Nx, Ny, Nz, h, order=0, mode="constant", cval=5)
    n = 5000
    zf = rng.random(n).astype(np.float32)
    zg = (0.7 * zf + 0.3 * rng.random(n)).astype(np.float32)
    zm = rng.random(n) < 0.6
    d.update(zf=zf, zg=zg, zm=zm, zncc=W.compute_zncc(zf, zg, zm),
             zncc_empty=W.compute_zncc(zf, zg, np.zeros(n, bool)))
    np.savez_compressed(os.path.join(OUT, "post.npz"), **d)


def prep_cases():
    """Preprocess glue (preprocess.py): bin_volume and compute_crop run from
    the reference module, imported with stand-ins for its module-level CuPy
    and tifffile imports (neither function uses them)."""
    import types
    for name in ("cupy", "tifffile"):
        sys.modules.setdefault(name, types.ModuleType(name))
    from voxeldvc import preprocess as P
    rng = np.random.default_rng(41)
    vol8 = rng.integers(0, 256, (12, 8, 16), dtype=np.uint8)
    volf = rng.random((9, 6, 12)).astype(np.float32) * 100
    f = _texture((40, 33, 29), rng).astype(np.float32)
    g = _texture((40, 33, 29), rng).astype(np.float32)
    f[:3] = 0.0
    g[:, -5:] = 0.0
    g[..., :2] = 0.0
    lo, hi = P.compute_crop(f, g, 4)
    lo2, hi2 = P.compute_crop(f, g, 8, glt=0.3)
    np.savez_compressed(os.path.join(OUT, "prep.npz"), vol8=vol8, volf=volf, bin8_2=P.bin_volume(vol8, 2),
                        bin8_4=P.bin_volume(vol8, 4), binf_3=P.bin_volume(volf, 3), f=f, g=g, lo=lo, hi=hi,
                        lo2=lo2, hi2=hi2)


def cells_cases():
    """Per-element output fields (engine/write_output.py:256-491) and the
    diagnostic masks (engine/kernels_dvc.py:92-341), from the reference
    functions, on two meshes."""
    from voxeldvc.engine import write_output as W
    rng = np.random.default_rng(53)
    d = {}
    for tag, (Nx, Ny, Nz, h) in (("a", (7, 6, 5, 3)), ("b", (6, 8, 7, 2)), ("c", (10, 11, 9, 1))):
        shape = (Nx * h + 1, Ny * h + 1, Nz * h + 1)
        Nn = (Nx + 1) * (Ny + 1) * (Nz + 1)
        U = rng.standard_normal(3 * Nn) * 0.3
        U_grid = np.stack([U[c::3].reshape(Nx + 1, Ny + 1, Nz + 1, order="F") for c in range(3)], axis=-1)
        ref = (_texture(shape, rng) * 40 + 60).astype(np.float32)
        ref[: h + 2, : h + 1] = 0.0                      # a void corner: non-material cells
        ref[-h - 1:, :, -h - 1:] = 80.0                  # a flat slab: zero-variance cells
        glt = 30.0
        active = ref > glt
        active[:, -(h // 2 + 1):, :] = False             # lost overlap along one face
        for _ in range(3):                               # isolated dropouts
            active[tuple(rng.integers(h, n - h) for n in shape)] = False
        res = np.where(active, rng.standard_normal(shape) * 3.0, 0.0)
        res[-h - 1:, :, -h - 1:] = np.where(active[-h - 1:, :, -h - 1:], 1.5, 0.0)
        res_flat = res.reshape(-1, order="F")
        active_flat = res_flat != 0
        mask0_flat = ref.reshape(-1, order="F") > glt
        unsafe = KD.compute_unsafe_voxel_mask(active_flat, h, Nx, Ny, Nz)
        dU = rng.standard_normal(3 * Nn) * 1e-3
        U0 = U.copy()
        for n in (0, 1, Nx + 1, Nx + 2, (Nx + 1) * (Ny + 1), (Nx + 1) * (Ny + 1) + 1,
                  (Nx + 1) * (Ny + 1) + Nx + 1, (Nx + 1) * (Ny + 1) + Nx + 2):
            U0[3 * n:3 * n + 3] = 0.0                    # element 0's corners: ||U|| = 0
        ps = W.compute_principal_strains_cell(U_grid, h)
        mat = W.compute_material_cell_mask(ref, h, Nx, Ny, Nz, glt=glt)
        # no cell mean within rounding of the threshold (float32 vs float64 sums)
        from voxeldvc.engine.kernels_dvc import get_voxel_offsets, get_elem_voxel_origins
        vox = get_elem_voxel_origins(np.arange(Nx * Ny * Nz), h, Nx, Ny, np)[:, None] + \
            get_voxel_offsets(h, Nx, Ny, np)[None, :]
        means = ref.reshape(-1, order="F").astype(np.float64)[vox].mean(axis=1)
        assert np.min(np.abs(means - glt)) > 1e-3 and np.min(np.abs(means - 70.0)) > 1e-3
        rstd, zn = W.compute_correlation_quality_cell(res_flat, ref, h, Nx, Ny, Nz)
        d.update({
            f"{tag}_dims": np.array([Nx, Ny, Nz, h]), f"{tag}_U": U, f"{tag}_U_grid": U_grid, f"{tag}_ref": ref,
            f"{tag}_glt": np.float64(glt), f"{tag}_res": res_flat, f"{tag}_mask0": mask0_flat,
            f"{tag}_dU": dU, f"{tag}_U0": U0,
            f"{tag}_principal": ps, f"{tag}_equivalent": W.compute_equivalent_strain(ps),
            f"{tag}_material": mat,
            f"{tag}_material70": W.compute_material_cell_mask(ref, h, Nx, Ny, Nz, glt=70.0), f"{tag}_material_eroded": W.compute_material_cell_mask_eroded(mat),
            f"{tag}_unsafe_vox": unsafe, f"{tag}_safe": W.compute_safe_cell_mask(unsafe, h, Nx, Ny, Nz),
            f"{tag}_unsafe_elem": KD.compute_unsafe_element_mask(active_flat, h, Nx, Ny, Nz),
            f"{tag}_unsafe_node": KD.compute_unsafe_node_mask(active_flat, h, Nx, Ny, Nz),
            f"{tag}_overlap_lost": KD.compute_overlap_lost_element_mask(active_flat, mask0_flat, h, Nx, Ny, Nz),
            f"{tag}_overlap_lost_t": KD.compute_overlap_lost_element_mask(active_flat, mask0_flat, h, Nx, Ny, Nz,
                                                                          frac_threshold=0.2,
                                                                          min_material_frac=0.3),
            f"{tag}_boundary": KD.boundary_element_mask(Nx, Ny, Nz),
            f"{tag}_residual_std": rstd, f"{tag}_zncc": zn,
            f"{tag}_gn": W.compute_gn_convergence_cell(dU, U0, Nx, Ny, Nz),
        })
        # an eroded mask with holes (interior non-material cells)
        holes = rng.random((Nx, Ny, Nz)) > 0.15
        d[f"{tag}_holes"] = holes
        d[f"{tag}_holes_eroded"] = W.compute_material_cell_mask_eroded(holes)
    ps3 = rng.standard_normal((7, 5, 3))
    d.update(ps3=ps3, eq3=W.compute_equivalent_strain(ps3))
    np.savez_compressed(os.path.join(OUT, "cells.npz"), **d)


def gt_cases():
    """Ground-truth harness (ground_truth/prepare_ground_truth.py,
    analyse_ground_truth.py): the backward warp with linear extrapolation,
    the uniaxial field, voxel recoverability, node support fractions and
    the grid -> DOF flattening, from the reference functions."""
    from voxeldvc.ground_truth import prepare_ground_truth as PG
    from voxeldvc.ground_truth import analyse_ground_truth as AG
    rng = np.random.default_rng(61)
    n = 17
    ref = _texture((n, n, n), rng) * 1000.0
    u = rng.standard_normal((n, n, n, 3)) * 1.5
    u[:3] += 2.5                                   # samples past the low x edge: extrapolation
    u[..., -2:, 2] -= 3.0                          # and past the high z edge
    u[5, 6, 7] = 0.0                               # an exact grid point
    u[8, 8, 8] = (0.5, -0.25, 1.0)                 # half-integers
    deformed = PG.make_deformed_image(ref, u)
    uni = PG.make_uniaxial_gt(9, 0.02)
    g_shape = (15, 19, 14)
    inb = AG.voxel_in_bounds(u, g_shape)
    h, nb, crop_lo = 4, (3, 4, 3), np.array([1, 0, 2])
    oob = AG.node_oob_fraction(u, h, *nb, g_shape, crop_lo)
    U_grid = rng.standard_normal((4, 3, 5, 3))
    np.savez_compressed(os.path.join(OUT, "gt.npz"), ref=ref, u=u, deformed=deformed, uni=uni,
                        g_shape=np.array(g_shape), inb=inb, h=np.int64(h), nb=np.array(nb), crop_lo=crop_lo,
                        oob=oob, U_grid=U_grid, dofs=AG.grid_to_dofs(U_grid))


def gt_pipeline_case(kind="z+0.01"):
    """The known-answer pipeline run through the reference's own CPU code
    on the seeded stand-in dataset (voxeldvc_gb300.synth.gt_stand_in):
    prepare (make_deformed_image), preprocess (affine_prealign,
    affine_refine_gn, compute_crop; the crop's warp onto the reference grid
    uses the oracle's restatement, the reference's needs CuPy), run
    (multiscale_correlate_gpu with NumPy, ext_affine seed), and the
    analysis (node / voxel errors over the recoverable and valid sets)."""
    import hashlib
    import types
    for name in ("cupy", "tifffile"):
        sys.modules.setdefault(name, types.ModuleType(name))
    sys.path.insert(0, os.path.dirname(os.path.dirname(OUT)))
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(OUT))))
    from voxeldvc_gb300.synth import gt_stand_in
    from oracle import dvc_oracle as O
    from voxeldvc import preprocess as P
    from voxeldvc.ground_truth import prepare_ground_truth as PG
    from voxeldvc.ground_truth import analyse_ground_truth as AG
    from voxeldvc.engine import write_output as W
    ref, U_in = gt_stand_in(kind)
    digest = hashlib.sha256(ref.tobytes() + U_in.tobytes()).hexdigest()
    n = ref.shape[0]
    u_vox = U_in.astype(np.float64)[:n, :n, :n]
    deformed = PG.make_deformed_image(ref.astype(np.float64), u_vox)
    h, glt, l0 = 8, 0.0, 4.5 * 8
    f_pix, g_pix = ref.astype(np.float32), deformed.astype(np.float32)
    A, t, c, info = CG.affine_prealign(f_pix, g_pix, np, decimate=4)
    A, t, rinfo = CG.affine_refine_gn(f_pix, g_pix, np, A, t, c)
    g_warped = O.warp_onto_ref_grid(A, t, c, ref.shape, g_pix)
    lo, hi = P.compute_crop(ref, g_warped, h, glt)
    corners = np.array([[lo[0] + dx * (hi[0] - lo[0] - 1), lo[1] + dy * (hi[1] - lo[1] - 1),
                         lo[2] + dz * (hi[2] - lo[2] - 1)] for dx in (0, 1) for dy in (0, 1) for dz in (0, 1)],
                       dtype=np.float64)
    cd = (corners - c) @ A.T + c + t
    lo_def = np.maximum(np.floor(cd.min(axis=0)).astype(int) - 1, 0)
    hi_def = np.minimum(np.ceil(cd.max(axis=0)).astype(int) + 2, np.array(deformed.shape))
    ref_c = ref[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]]
    def_c = deformed[lo_def[0]:hi_def[0], lo_def[1]:hi_def[1], lo_def[2]:hi_def[2]]
    Nx, Ny, Nz = ((s - 1) // h for s in ref_c.shape)
    U, res, dU = CG.multiscale_correlate_gpu(ref_c, def_c, Nx, Ny, Nz, h, xp=np, scales=(2, 1, 0), l0=l0, glt=glt,
                                             K_ref_laplacian=G.build_K_ref_laplacian(), dynamic_mask=True,
                                             fft_prealign=False, prealign_affine=False,
                                             ext_affine=(A, t + lo - lo_def, c - lo), disp=False,
                                             freeze_mask_after=4)
    nb = (Nx + 1, Ny + 1, Nz + 1)
    U_grid = np.stack([U[k::3].reshape(nb, order="F") for k in range(3)], axis=-1) + lo_def - lo
    u_nodes = u_vox[np.ix_(*(lo[a] + np.arange(nb[a]) * h for a in range(3)))]
    err = U_grid - u_nodes
    oob = AG.node_oob_fraction(u_vox, h, *nb, deformed.shape, lo)
    rec = oob <= 0
    active = CG.compute_active_mask(U + np.tile(lo_def, len(U) // 3), def_c, Nx, Ny, Nz, h, np,
                                    g_origin=tuple(int(x) for x in lo_def), mask0_vox=ref_c.reshape(-1, order="F") > glt,
                                    glt=glt)
    active = np.asarray(active)
    lost = KD.compute_overlap_lost_element_mask(active, ref_c.reshape(-1, order="F") > glt, h, Nx, Ny, Nz)
    node_idx = G.build_node_index(Nx, Ny, Nz)
    en = G.element_node_ids(node_idx, Nx, Ny, Nz)
    nm = np.zeros(node_idx.size, bool)
    nm[en[lost].ravel()] = True
    valid = rec & ~nm[node_idx]
    rms = lambda m: float(np.sqrt(np.mean(err[m] ** 2)))  # noqa: E731
    np.savez_compressed(os.path.join(OUT, f"gt_pipeline_{kind}.npz"), digest=np.array(digest), A=A, t=t, c=c,
                        lo=lo, hi=hi, lo_def=lo_def, hi_def=hi_def, U_grid=U_grid, err=err, rec=rec,
                        valid=valid, rms_rec=rms(rec), rms_valid=rms(valid), rms_all=rms(np.ones_like(rec)))
    print(kind, "recoverable RMS", rms(rec), "valid RMS", rms(valid), "nodes", rec.sum(), valid.sum())
    del W


RUN_SETTINGS = dict(dynamic_mask=True, freeze_mask_after=4, maxiter=30, eps=1e-3, pcg_tol=1e-6, pcg_max_iter=2000,
                    glt=0.0, fft_prealign=True, scales=(2, 1, 0))


def baseline_solve(case="plain_small", reg="laplacian", dtype="float32", scales=""):
    """One benchmark-family workload solved by the reference's own
    `multiscale_correlate_gpu` on NumPy with the `voxeldvc run` settings
    (correlate_gpu.py:1143-1305): inputs from `workload_inputs` (regenerated
    from seeds by the tests; their digest is stored), the nodal U, per
    pyramid level the GN iteration count, the dU/U log and the PCG
    iteration count of every GN iteration (the reference's `pcg` calls its
    matvec once for the initial residual and once per iteration), and the
    CPU wall time of the solve.

    case: plain_small (129^3, h = 16, Laplacian l0 = 2 h) or necking_129 /
    necking_257 / necking_513 (h = 8, l0 = 4.5 h; reg laplacian or
    equilibrium_gap with nu = 0.3, reg_exponent 4).  scales: pyramid levels
    to run, e.g. "2" for the coarsest level alone (with its FFT seed),
    default 2/1/0."""
    import contextlib
    import io
    import re
    import time
    sys.path.insert(0, os.path.dirname(os.path.dirname(OUT)))
    from oracle import workload_inputs as WI
    f, g = WI.CASES[case]()
    h = 16 if case == "plain_small" else 8
    Nx, Ny, Nz = ((s - 1) // h for s in f.shape)
    kw = dict(RUN_SETTINGS, K_ref_laplacian=G.build_K_ref_laplacian(), l0=(2.0 if case == "plain_small" else 4.5) * h,
              dtype=np.dtype(dtype).type, disp=True)
    if reg == "equilibrium_gap":
        kw.update(reg_type="equilibrium_gap", K_ref_elastic=G.build_K_ref(0.3), reg_exponent=4)
    if scales:
        kw["scales"] = tuple(int(c) for c in scales.split("/"))
    pcg_counts = []
    real_pcg = CG.pcg

    def counting_pcg(matvec, *a, **k):
        n = [0]

        def mv(v):
            n[0] += 1
            return matvec(v)
        x = real_pcg(mv, *a, **k)
        pcg_counts.append(n[0] - 1)
        return x

    CG.pcg = counting_pcg
    buf = io.StringIO()
    try:
        t0 = time.perf_counter()
        with contextlib.redirect_stdout(buf):
            U, res, dU = CG.multiscale_correlate_gpu(f, g, Nx, Ny, Nz, h, xp=np, **kw)
        wall = time.perf_counter() - t0
    finally:
        CG.pcg = real_pcg
    log = buf.getvalue()
    levels, errs = [], []
    for line in log.splitlines():
        if line.startswith("=== MULTISCALE"):
            levels.append([])
        m = re.search(r"dU/U=([0-9.eE+-]+|nan|inf)", line)
        if m and levels:
            levels[-1].append(float(m.group(1)))
    gn = [len(lv) for lv in levels]
    pcg, k = [], 0
    for n in gn:
        pcg.append(pcg_counts[k:k + n])
        k += n
    tag = f"{case}_{'lap' if reg == 'laplacian' else 'eqgap'}_{'f64' if dtype == 'float64' else 'f32'}"
    if scales:
        tag += "_s" + scales.replace("/", "")
    np.savez_compressed(os.path.join(OUT, f"baseline_{tag}.npz"), digest=np.array(WI.digest(f, g)),
                        dims=np.array([Nx, Ny, Nz, h]), U=U if U.size < 200_000 else U.astype(np.float32), res_sumsq=np.float64(np.sum(np.square(res, dtype=np.float64))),
                        gn_iters=np.array(gn), pcg_iters=np.array(pcg_counts), du_log=np.array(sum(levels, [])),
                        wall_s=np.float64(wall), reg=np.array(reg), l0=np.float64(kw["l0"]),
                        scales=np.array(kw["scales"]),
                        log=np.array(log))
    print(tag, "wall", round(wall, 1), "s; GN", gn, "PCG", pcg, "dU/U", [lv[-1] if lv else None for lv in levels])


if __name__ == "__main__":
    if len(sys.argv) > 1:  # regenerate only the named case groups: name[:arg,arg...]
        for spec in sys.argv[1:]:
            name, _, rest = spec.partition(":")
            globals()[name](*(rest.split(",") if rest else ()))
        sys.exit(0)
    gt_cases()
    cells_cases()
    prep_cases()
    post_cases()
    affine_cases()
    geometry()
    operators("A", 3, 2, 2, 4, seed=1)
    operators("B", 2, 3, 1, 3, seed=2)
    operators("C", 1, 1, 1, 2, seed=3)
    operators("D", 4, 3, 2, 8, seed=4)
    operators("E", 5, 1, 2, 1, seed=8)
    solves()
    fft_cases()
    for fn in sorted(os.listdir(OUT)):
        if fn.endswith(".npz"):
            print(fn, os.path.getsize(os.path.join(OUT, fn)))
