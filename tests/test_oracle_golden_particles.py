"""The oracle's particle preparation against the reference's own
ParticleFourierPreparer.prepare (v606:1321-1374) at boxes the stage fixtures
do not cover: 96, 192 cropped to 96 in Fourier space, and 256
(tests/golden/make_golden_particles.py; inputs regenerated from its seeds)."""
import sys
from pathlib import Path

import numpy as np
import pytest

from oracle import gisapr_oracle as O
from tests.helpers import SPECTRUM_RRMS, rrms

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
from make_golden_particles import case_inputs  # noqa: E402

GOLDEN = Path(__file__).resolve().parent / "golden" / "golden_particles.npz"


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


@pytest.mark.parametrize("k", range(3))
def test_oracle_particle_spectra_match_reference(golden, k):
    n, nb, radius, edge, seed = (int(v) for v in golden[f"case{k}"])
    image, weights, angles = case_inputs(n, nb, seed)
    spec = O.prepare_particle(image, angles, weights, O.soft_mask(n, radius, edge), nb)
    ref = golden[f"spectra{k}"]
    assert spec.shape == (3, nb, nb // 2 + 1) and ref.shape[0] == 3 and ref.shape[2] == nb // 2 + 1
    assert rrms(spec[:, :ref.shape[1]], ref) < SPECTRUM_RRMS     # measured 2.4e-7 to 1.8e-6
    # every psi angle's spectrum has unit norm, as the reference's
    np.testing.assert_allclose(np.sqrt((np.abs(spec) ** 2).sum(axis=(1, 2))), golden[f"norms{k}"], atol=1e-5)
