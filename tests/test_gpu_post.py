"""Post-solve voxel stages on the GPU against the reference's own outputs
(tests/golden/post.npz): push_field_forward in both orders and modes, on
float and label fields, and compute_zncc."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def W(cuda):
    from voxeldvc_gb300.engine import write_output
    return write_output


CASES = (("o1_nearest", dict(order=1, mode="nearest")),
         ("o1_constant", dict(order=1, mode="constant", cval=-1.0)),
         ("o0_constant", dict(order=0, mode="constant", cval=7.0)))


@pytest.mark.parametrize("name", ["f32", "f64"])
def test_push_field_forward(W, name):
    c = load_golden("post.npz")
    Nx, Ny, Nz, h = (int(x) for x in c["dims"])
    for key, kw in CASES:
        out = W.push_field_forward(c[name], c["U"], Nx, Ny, Nz, h, **kw)
        ref = c[f"{name}_{key}"]
        assert out.shape == ref.shape and out.dtype == ref.dtype
        if kw["order"] == 0:
            assert np.array_equal(out, ref), key
        else:
            tol = 2e-7 if name == "f32" else 1e-13
            assert np.allclose(out, ref, rtol=tol, atol=tol), key


def test_push_label_field_and_reference_alias(W):
    c = load_golden("post.npz")
    Nx, Ny, Nz, h = (int(x) for x in c["dims"])
    out = W.push_field_forward(c["lab"], c["U"], Nx, Ny, Nz, h, order=0, mode="nearest")
    assert out.dtype == np.uint8 and np.array_equal(out, c["lab_o0_nearest"])
    out = W.push_field_forward(c["lab"], c["U"], Nx, Ny, Nz, h, order=0, mode="constant", cval=5)
    assert np.array_equal(out, c["lab_o0_constant"])
    ref = W.push_reference_forward(c["f64"], c["U"], Nx, Ny, Nz, h)
    assert np.allclose(ref, c["f64_o1_nearest"], rtol=1e-13, atol=1e-13)
    with pytest.raises(ValueError):
        W.push_field_forward(c["f64"][:-1], c["U"], Nx, Ny, Nz, h)
    with pytest.raises(ValueError):
        W.push_field_forward(c["f64"], c["U"], Nx, Ny, Nz, h, mode="wrap")


def test_push_integer_fields_round_like_the_sampler(W):
    """Order-1 pushes of integer fields round half away from zero, as the
    reference's sampler converts to an integer output."""
    c = load_golden("post.npz")
    Nx, Ny, Nz, h = (int(x) for x in c["dims"])
    out = W.push_field_forward(c["u16"], c["U"], Nx, Ny, Nz, h, order=1)
    assert out.dtype == np.uint16 and np.array_equal(out, c["u16_o1_nearest"])
    out = W.push_field_forward(c["lab"] * 40, c["U"], Nx, Ny, Nz, h, order=1)
    assert out.dtype == np.uint8 and np.array_equal(out, c["lab_o1_nearest"])


def test_compute_zncc(W):
    c = load_golden("post.npz")
    assert W.compute_zncc(c["zf"], c["zg"], c["zm"]) == pytest.approx(float(c["zncc"]), abs=1e-13)
    assert np.isnan(W.compute_zncc(c["zf"], c["zg"], np.zeros_like(c["zm"])))
