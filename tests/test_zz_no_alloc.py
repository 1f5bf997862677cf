"""vdvc_matvec_H_noalloc: the Hessian matvec for callers that cannot allocate
device memory (a plugin whose host application owns all device memory
through its own pool, or a latency-critical loop where cudaMalloc is not
allowed).  Its scratch is a fixed file-scope device array instead of a
caller workspace; the result must equal vdvc_matvec_H's.

This file sorts last so that a run stopping at its first failure has
already run every other test.  It passes on its own in a fresh process too.
"""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

RTOL = 5e-6  # the float32 operator tolerance used by the other GPU tests


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("case", ["A", "B", "D"])
def test_noalloc_matches_workspace_entry_point_twice(cuda, case):
    torch = cuda
    from voxeldvc_gb300 import _lib
    L = _lib.lib()
    c = load_golden(f"ops_{case}.npz")
    Nx, Ny, Nz, h = (int(x) for x in c["dims"])
    v = torch.from_numpy(c["v"]).cuda()
    g = torch.from_numpy(c["grad"]).cuda()
    m = torch.from_numpy(c["mask"]).cuda()
    s = torch.cuda.current_stream().cuda_stream
    ref = torch.empty_like(v)
    nws = L.vdvc_workspace_bytes(_lib.F32, h, Nx, Ny, Nz)
    ws = torch.empty(nws, dtype=torch.uint8, device="cuda")
    assert L.vdvc_matvec_H(v.data_ptr(), g.data_ptr(), m.data_ptr(), _lib.F32, h, Nx, Ny, Nz, ref.data_ptr(),
                           ws.data_ptr(), nws, s) == _lib.OK
    ref_h = ref.cpu().numpy()
    for call in range(2):  # the shared scratch keeps the previous call's contents
        out = torch.full_like(v, float("nan"))
        st = L.vdvc_matvec_H_noalloc(v.data_ptr(), g.data_ptr(), m.data_ptr(), h, Nx, Ny, Nz, out.data_ptr(), s)
        assert st == _lib.OK, _lib.last_error()
        o = out.cpu().numpy()
        assert np.all(np.isfinite(o))
        assert rel(o, ref_h) <= RTOL, f"call {call}"
        assert rel(o, c["out_matvec_H"]) < RTOL


def test_noalloc_rejects_meshes_beyond_its_scratch(cuda):
    torch = cuda
    from voxeldvc_gb300 import _lib
    L = _lib.lib()
    cap = L.vdvc_matvec_H_noalloc_max_elements()
    assert cap == (32 << 20) // 96
    c = load_golden("ops_A.npz")
    v = torch.from_numpy(c["v"]).cuda()
    # 80^3 elements of h = 1 need 49 MB of element vectors: refused before any device work
    st = L.vdvc_matvec_H_noalloc(v.data_ptr(), v.data_ptr(), v.data_ptr(), 1, 80, 80, 80, v.data_ptr(),
                                 torch.cuda.current_stream().cuda_stream)
    assert st == _lib.ERR_ARG
    assert "at most" in _lib.last_error()


def test_noalloc_makes_no_device_allocation(cuda):
    """After its first call on a device (which looks up the scratch array's
    address), the entry point allocates no device memory: the device's free
    memory is the same before and after further calls."""
    torch = cuda
    from voxeldvc_gb300 import _lib
    L = _lib.lib()
    c = load_golden("ops_D.npz")
    Nx, Ny, Nz, h = (int(x) for x in c["dims"])
    v = torch.from_numpy(c["v"]).cuda()
    g = torch.from_numpy(c["grad"]).cuda()
    m = torch.from_numpy(c["mask"]).cuda()
    out = torch.empty_like(v)
    s = torch.cuda.current_stream().cuda_stream

    def call():
        st = L.vdvc_matvec_H_noalloc(v.data_ptr(), g.data_ptr(), m.data_ptr(), h, Nx, Ny, Nz, out.data_ptr(), s)
        assert st == _lib.OK, _lib.last_error()

    call()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        call()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert rel(out.cpu().numpy(), c["out_matvec_H"]) < RTOL
