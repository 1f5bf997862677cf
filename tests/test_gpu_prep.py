"""Preprocess glue on the GPU (voxeldvc_gb300.preprocess) against the
reference's own bin_volume / compute_crop outputs and the warp oracle."""
import numpy as np
import pytest

from conftest import load_golden
from oracle import dvc_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P(cuda):
    from voxeldvc_gb300 import preprocess
    return preprocess


def test_bin_volume(P):
    c = load_golden("prep.npz")
    assert np.array_equal(P.bin_volume(c["vol8"], 2), c["bin8_2"])
    assert np.array_equal(P.bin_volume(c["vol8"], 4), c["bin8_4"])
    assert np.array_equal(P.bin_volume(c["volf"], 3), c["binf_3"])
    v16 = (np.arange(6 * 4 * 8) * 1000 % 65521).astype(np.uint16).reshape(6, 4, 8)
    assert np.array_equal(P.bin_volume(v16, 2), O.bin_volume(v16, 2))
    with pytest.raises(AssertionError):
        P.bin_volume(c["vol8"], 5)


def test_compute_crop(P):
    c = load_golden("prep.npz")
    lo, hi = P.compute_crop(c["f"], c["g"], 4)
    assert np.array_equal(lo, c["lo"]) and np.array_equal(hi, c["hi"])
    lo, hi = P.compute_crop(c["f"], c["g"], 8, glt=0.3)
    assert np.array_equal(lo, c["lo2"]) and np.array_equal(hi, c["hi2"])
    with pytest.raises(RuntimeError):
        P.compute_crop(c["f"], np.zeros_like(c["g"]), 4)


def test_warp_onto_ref_grid(P):
    c = load_golden("prep.npz")
    g = c["f"]
    rng = np.random.default_rng(3)
    th = np.deg2rad(4.0)
    A = np.array([[np.cos(th), -np.sin(th), 0.0], [np.sin(th), np.cos(th), 0.0], [0.0, 0.0, 1.02]])
    t = np.array([1.3, -0.7, 2.1])
    cc = np.array(g.shape, float) / 2
    Nf = (36, 30, 27)
    out = P.warp_onto_ref_grid(A, t, cc, Nf, g, np)
    ref = O.warp_onto_ref_grid(A, t, cc, Nf, g)
    assert out.shape == Nf and out.dtype == np.float32
    assert np.abs(out - ref).max() < 1e-5 * np.abs(ref).max()
    ident = P.warp_onto_ref_grid(np.eye(3), np.zeros(3), cc, g.shape, g, np)
    assert np.array_equal(ident, g)
    sh = P.warp_onto_ref_grid(np.eye(3), np.array([2.0, 0.0, -1.0]), np.zeros(3), g.shape, g, np)
    assert np.array_equal(sh[:-2, :, 1:], g[2:, :, :-1]) and np.all(sh[-2:] == 0)
