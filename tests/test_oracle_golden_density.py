"""The oracle's Gaussian splat against the reference's own
density_from_coords (R/pdb2mrc_gpu_ver_fp32_v3.py:41-98) at box 256 / 0.85 A
(the precision configuration) and box 96 / 1.4 A, atoms over the whole box
including its faces (tests/golden/make_golden_density.py; coordinates
regenerated from its seeds)."""
import sys
from pathlib import Path

import numpy as np
import pytest

from oracle import gisapr_oracle as O
from tests.helpers import DENSITY_RRMS, rrms

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
from make_golden_density import CASES, case_atoms, planes  # noqa: E402

GOLDEN = Path(__file__).resolve().parent / "golden" / "golden_density.npz"


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


@pytest.mark.parametrize("k", range(len(CASES)))
def test_oracle_density_matches_reference(golden, k):
    n, apix, res, n_atoms, seed = CASES[k]
    xyz, z = case_atoms(n, apix, n_atoms, seed)
    d = np.asarray(O.splat_density(xyz, z, n, apix, res))
    d64 = d.astype(np.float64)
    # whole-volume sums and three planes (measured 6e-9 and 8e-8 relative)
    np.testing.assert_allclose([d64.sum(), (d64 * d64).sum()], golden[f"sums{k}"], rtol=1e-7)
    assert rrms(d[planes(n)], golden[f"planes{k}"]) < DENSITY_RRMS
