"""Whole multiscale solves of the benchmark workload family on the GPU
against the reference's own NumPy solve of the same inputs
(tests/golden/baseline_*.npz, written by make_golden.py::baseline_solve with
the `voxeldvc run` settings: dynamic mask frozen after 4 iterations,
maxiter 30, eps 1e-3, PCG tol 1e-6 / 2000 iterations, glt 0, FFT seed):

  * plain_small: 129^3, 200 cylinders, 1 % z strain + translation, h = 16,
    Laplacian l0 = 2 h, scales (2, 1, 0), in FP32 and FP64;
  * necking_129 / necking_257: replicas of the 513^3 tensile-necking
    workload, h = 8, Laplacian l0 = 4.5 h, scales (2, 1, 0);
  * necking_513 at scale 2 alone: the coarsest pyramid level of the 513^3
    benchmark workload itself (129^3 voxels, h = 2, 64^3 elements) with its
    FFT seed.

The inputs are regenerated from their seeds by oracle/workload_inputs.py
(the golden stores the digest of the bytes the reference saw).  Bars: nodal
U within 1e-3 vx RMS of the reference at FP32 (1e-4 at FP64), the same GN
iteration count on every pyramid level, and every GN iteration's PCG count
within one of the reference's (the reference runs its PCG in float64 once
b is promoted by the regularizer term; the FP32 solve runs FP32 vectors).

necking_129 with the equilibrium-gap regularizer (nu 0.3, exponent 4) at
scale 2 is the reference's own evidence that this regularizer does not
converge on the benchmark family: its solve runs all 30 GN iterations, its
PCG reaches the 2000-iteration cap from the third GN iteration on, and dU/U
stalls near 0.1.  Such a solve is chaotic in its rounding (PCG capped every
iteration), so the bar there is the same behaviour: GN at the cap, the
first GN iteration's PCG count within 5 %, the PCG cap reached as often,
dU/U never below 10 eps.
"""
import glob
import os
import warnings

import numpy as np
import pytest

from conftest import GOLDEN, load_golden

pytestmark = pytest.mark.gpu

CASES = sorted(os.path.basename(p) for p in glob.glob(os.path.join(GOLDEN, "baseline_*.npz")))


def rms(a, b):
    return float(np.sqrt(np.mean((np.asarray(a, np.float64) - np.asarray(b, np.float64)) ** 2)))


@pytest.mark.parametrize("name", CASES)
def test_baseline_solve(cuda, name):
    from oracle import workload_inputs as WI
    from voxeldvc_gb300.engine import correlate_gpu as CG, geometry_dvc as G
    gold = load_golden(name)
    case = name[len("baseline_"):].split("_lap")[0].split("_eqgap")[0]
    f, g = WI.CASES[case]()
    if WI.digest(f, g) != str(gold["digest"]):
        warnings.warn(f"{case}: regenerated inputs differ in their last bits from the reference's "
                      "(different NumPy/SciPy build); compared within the tolerances all the same")
    Nx, Ny, Nz, h = (int(x) for x in gold["dims"])
    f64 = name.endswith("_f64.npz") or "_f64_" in name
    kw = dict(dynamic_mask=True, freeze_mask_after=4, maxiter=30, eps=1e-3, pcg_tol=1e-6, pcg_max_iter=2000,
              glt=0.0, fft_prealign=True, scales=tuple(int(s) for s in gold["scales"]),
              K_ref_laplacian=G.build_K_ref_laplacian(), l0=float(gold["l0"]), disp=False,
              dtype=np.float64 if f64 else np.float32)
    if str(gold["reg"]) == "equilibrium_gap":
        kw.update(reg_type="equilibrium_gap", K_ref_elastic=G.build_K_ref(0.3), reg_exponent=4)
    stats = []
    U, res, dU = CG.multiscale_correlate_gpu(f, g, Nx, Ny, Nz, h, xp=np, stats=stats, **kw)
    gn = [s["gn_iters"] for s in stats]
    pcg = sum((list(s["pcg_iters"]) for s in stats), [])
    if str(gold["reg"]) == "equilibrium_gap":
        ref_pcg = np.asarray(gold["pcg_iters"])
        du = np.asarray(sum((list(s["du"]) for s in stats), []))
        assert gn == [int(x) for x in gold["gn_iters"]] == [kw["maxiter"]] * len(gn), (gn, gold["gn_iters"])
        assert abs(pcg[0] - ref_pcg[0]) <= 0.05 * ref_pcg[0], (pcg[0], ref_pcg[0])
        capped, ref_capped = int(np.sum(np.asarray(pcg) == 2000)), int(np.sum(ref_pcg == 2000))
        assert abs(capped - ref_capped) <= 2, (capped, ref_capped)
        assert du.min() > 10 * kw["eps"] and np.asarray(gold["du_log"]).min() > 10 * kw["eps"]
        assert np.all(np.isfinite(U))
        return
    assert gn == [int(x) for x in gold["gn_iters"]], (gn, gold["gn_iters"])
    d = np.abs(np.array(pcg) - gold["pcg_iters"])
    assert d.max() <= 1, (pcg, gold["pcg_iters"].tolist())
    err = rms(U, gold["U"])
    assert err < (1e-4 if f64 else 1e-3), err
