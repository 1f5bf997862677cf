"""The seeded NumPy generator of the benchmark workload family
(oracle/workload_inputs.py) reproduces the bytes the reference's golden
solves were run on (tests/golden/baseline_*.npz store their digest), and
the goldens hold what the GPU parity tests read."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden

CASES = sorted(os.path.basename(p) for p in glob.glob(os.path.join(GOLDEN, "baseline_*.npz")))
FAST = ("plain_small", "necking_129", "necking_257")


def _case(name):
    return name[len("baseline_"):].split("_lap")[0].split("_eqgap")[0]


@pytest.mark.parametrize("name", [n for n in CASES if _case(n) in FAST])
def test_inputs_reproduce_digest(name):
    from oracle import workload_inputs as WI
    gold = load_golden(name)
    f, g = WI.CASES[_case(name)]()
    assert WI.digest(f, g) == str(gold["digest"])
    assert f.dtype == np.float32 and g.dtype == np.float32
    assert 0.0 <= float(f.min()) and float(f.max()) <= 1.0


@pytest.mark.parametrize("name", CASES)
def test_golden_contents(name):
    gold = load_golden(name)
    Nx, Ny, Nz, h = (int(x) for x in gold["dims"])
    assert gold["U"].shape == (3 * (Nx + 1) * (Ny + 1) * (Nz + 1),)
    assert len(gold["gn_iters"]) == len(gold["scales"])
    assert int(np.sum(gold["gn_iters"])) == len(gold["pcg_iters"]) == len(gold["du_log"])
    assert np.all(np.isfinite(gold["U"]))
