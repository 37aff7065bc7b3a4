"""The oracle's templates with a Fourier crop (new box below the box:
128 -> 64, 192 -> 96, 256 -> 128) against the reference's own projector
(tests/golden/make_golden_templates_crop.py; densities and directions
regenerated from its seeds)."""
import sys
from pathlib import Path

import numpy as np
import pytest

from gisapr_gb300 import synthetic as syn
from oracle import gisapr_oracle as O
from tests.helpers import rrms

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
from make_golden_templates_crop import APIX, CASES, MASK_EDGE, case_directions  # noqa: E402

GOLDEN = Path(__file__).resolve().parent / "golden" / "golden_templates_crop.npz"


@pytest.fixture(scope="module")
def golden():
    return dict(np.load(GOLDEN))


@pytest.mark.parametrize("k", range(len(CASES)))
def test_oracle_cropped_templates_match_reference(golden, k):
    n, nb, n_dir, half_res, seed = CASES[k]
    radius = int(golden[f"case{k}"][5])
    rot, tilt = case_directions(n_dir, seed)
    mask = O.soft_mask(n, radius, MASK_EDGE)
    fsc = syn.logistic_fsc(n, APIX, half_res)
    packed_fsc = np.ascontiguousarray(O.centered_to_packed(O.radial_map(fsc, nb)))
    dft = O.volume_spectrum(syn.blob_density(n, seed))
    rot_t = O.rotation_matrices_t(rot, tilt)
    want = golden[f"templates{k}"]
    assert want.shape == (n_dir, nb, nb // 2 + 1)
    for j in range(n_dir):
        got = O.template_from_slice(O.central_slice(dft, rot_t[j], n), n, nb, mask, packed_fsc)
        # float64 oracle against the reference's float32 arithmetic
        # (measured 2.2e-5 to 8.8e-5 relative RMS)
        assert rrms(got, want[j]) < 1e-4, (n, nb, j, rrms(got, want[j]))
