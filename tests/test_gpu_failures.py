"""Failure detection without a GPU fault.

* The library's bounded device-side wait (the mbarrier wait of the
  bulk-copy and tensor-core pipelines) is driven into a timeout by
  vdvc_selftest_bounded_wait -- an mbarrier nothing arrives at -- and must
  come back as VDVC_ERR_TIMEOUT with the CUDA context still usable.
* Host-side injections into the solve: a non-finite initial displacement
  (NaN in b through the regularizer term), unsupported nodes with no
  regularizer (a zero Jacobi diagonal), an empty mask (the reference's
  ZeroDivisionError, correlate_gpu.py:1095) and a forced PCG iteration cap.
"""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

POLLS = 20000  # a few milliseconds of polling


def _matvec_still_right(torch):
    from voxeldvc_gb300.engine import kernels_dvc as K, geometry_dvc as G
    c = load_golden("ops_A.npz")
    Nx, Ny, Nz, h = (int(x) for x in c["dims"])
    N, w = G.build_N_stencil(h)
    out = K.matvec_H(c["v"], c["grad"], c["mask"], N, w, h, Nx, Ny, Nz, np)
    ref = c["out_matvec_H"]
    assert np.linalg.norm(out - ref) / np.linalg.norm(ref) < 5e-6


def test_bounded_wait_times_out_and_context_survives(cuda):
    torch = cuda
    from voxeldvc_gb300 import _lib
    L = _lib.lib()
    s = torch.cuda.current_stream().cuda_stream
    st = L.vdvc_selftest_bounded_wait(0, POLLS, s)
    assert st == _lib.ERR_TIMEOUT, (st, _lib.last_error())
    assert "ran out" in _lib.last_error()
    with pytest.raises(_lib.VdvcTimeout):
        _lib.check(st, "self-test")
    torch.cuda.synchronize()
    # the same wait released normally, then real work, on the same context
    assert L.vdvc_selftest_bounded_wait(1, POLLS, s) == _lib.OK, _lib.last_error()
    _matvec_still_right(torch)


def test_selftest_rejects_bad_arguments(cuda):
    from voxeldvc_gb300 import _lib
    L = _lib.lib()
    assert L.vdvc_selftest_bounded_wait(2, POLLS, None) == _lib.ERR_ARG
    assert L.vdvc_selftest_bounded_wait(0, 0, None) == _lib.ERR_ARG


@pytest.fixture(scope="module")
def problem():
    c = load_golden("solve_dynamic.npz")
    return c["f"], c["g"]


def test_nonfinite_initial_field_reports_status(cuda, problem):
    """NaN in U0 makes b non-finite (b = ... - ll R U): the PCG stops at once
    with VDVC_ERR_NONFINITE and U comes back non-finite.  The next GN
    iteration then samples g at non-finite positions, its mask is empty and
    the solve raises ZeroDivisionError, as the reference's does
    (correlate_gpu.py:1095, std0 / std1 with std1 = 0).  A clean solve
    afterwards is unaffected."""
    from voxeldvc_gb300 import _lib
    from voxeldvc_gb300.engine import correlate_gpu as CG, geometry_dvc as G
    f, g = problem
    kw = dict(K_ref_laplacian=G.build_K_ref_laplacian(), l0=8.0, eps=1e-4, disp=False)
    U0 = np.zeros(3 * 5 ** 3)
    U0[7] = np.nan
    stats = []
    U, _, _ = CG.correlate_gpu(f, g, 4, 4, 4, 4, xp=np, U0=U0, stats=stats, maxiter=1, **kw)
    assert not np.all(np.isfinite(U))
    assert stats[0]["pcg_status"] == [_lib.ERR_NONFINITE] and stats[0]["pcg_iters"][0] <= 1
    with pytest.raises(ZeroDivisionError):
        CG.correlate_gpu(f, g, 4, 4, 4, 4, xp=np, U0=U0, maxiter=2, **kw)
    c = load_golden("solve_dynamic.npz")
    Uc, _, _ = CG.correlate_gpu(f, g, 4, 4, 4, 4, xp=np, K_ref_laplacian=G.build_K_ref_laplacian(), l0=8.0,
                                maxiter=12, eps=1e-4, disp=False, dynamic_mask=True, freeze_mask_after=2, glt=0.0)
    assert float(np.sqrt(np.mean((Uc.astype(np.float64) - c["U"]) ** 2))) < 1e-3


def test_zero_diagonal_without_regularizer(cuda):
    """No regularizer and a block of nodes whose elements hold no masked
    voxel: their Jacobi diagonal is 0, min(diag) = 0, so M^-1 is infinite
    there -- the reference's 1 / (diag + 1e-5 min diag) does the same -- and
    the PCG reports VDVC_ERR_NONFINITE instead of running on."""
    from voxeldvc_gb300 import _lib
    from voxeldvc_gb300.engine import correlate_gpu as CG
    rng = np.random.default_rng(3)
    n = 17
    f = (rng.random((n, n, n)) + 0.1).astype(np.float32)
    f[:9, :9, :9] = 0.0  # element (0,0,0)'s voxels and more: out of mask0
    g = np.roll(f, 1, axis=0)
    stats = []
    U, _, _ = CG.correlate_gpu(f, g, 4, 4, 4, 4, xp=np, maxiter=1, eps=1e-6, disp=False, stats=stats)
    assert stats[0]["pcg_status"] == [_lib.ERR_NONFINITE]
    assert not np.all(np.isfinite(U))


def test_empty_mask_raises_zero_division(cuda, problem):
    from voxeldvc_gb300.engine import correlate_gpu as CG
    f, _ = problem
    with pytest.raises(ZeroDivisionError):
        CG.correlate_gpu(f, np.zeros_like(f), 4, 4, 4, 4, xp=np, maxiter=2, disp=False)


def test_forced_pcg_iteration_cap(cuda, problem):
    """pcg_max_iter caps every PCG at exactly that many iterations (the
    reference returns its iterate after max_iter), with an OK status."""
    from voxeldvc_gb300 import _lib
    from voxeldvc_gb300.engine import correlate_gpu as CG, geometry_dvc as G
    f, g = problem
    stats = []
    U, _, _ = CG.correlate_gpu(f, g, 4, 4, 4, 4, xp=np, K_ref_laplacian=G.build_K_ref_laplacian(), l0=8.0,
                               maxiter=4, eps=1e-12, pcg_max_iter=3, pcg_tol=1e-30, disp=False, stats=stats)
    assert stats[0]["pcg_iters"] == [3, 3, 3, 3]
    assert all(s == _lib.OK for s in stats[0]["pcg_status"])
    assert np.all(np.isfinite(U))
