"""The oracle's crop-window correlation against the reference's own
correlate_templates_and_particle (v606:1418-1449) at the sizes and crops the
stage fixtures do not cover: box 256 with crop 14 (the precision
configuration's shapes), 192 with crop 10, 96 with crop 12 and 64 with crop 14
(tests/golden/make_golden_correlate.py; inputs regenerated from its seeds)."""
import sys
from pathlib import Path

import numpy as np
import pytest

from oracle import gisapr_oracle as O

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
from make_golden_correlate import case_inputs  # noqa: E402

from tests.helpers import TIE_REL  # noqa: E402

GOLDEN = Path(__file__).resolve().parent / "golden" / "golden_correlate.npz"


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


@pytest.mark.parametrize("k", range(4))
def test_oracle_correlation_matches_reference(golden, k):
    n, crop, n_psi, n_t, seed = (int(v) for v in golden[f"case{k}"])
    t, p = case_inputs(n, n_psi, n_t, seed)
    raw = O.correlation_window(t, p, crop)                       # FP64 maps [n_t][n_psi][crop][crop]
    s, y, x = O.correlate(t, p, crop)
    ref_s, ref_y, ref_x = golden[f"scores{k}"], golden[f"ys{k}"], golden[f"xs{k}"]
    assert ref_s.shape == s.shape == (n_t, n_psi)
    # the reference's float32 maxima against the FP64 ones, relative to the map scale
    scale = np.abs(raw).max(axis=(2, 3)) * 1024.0
    assert np.max(np.abs(s - ref_s) / scale) < 1e-6  # measured 0.7-1.8e-7
    # positions identical, or the reference's position a tie of the FP64 maximum
    for a in range(n_t):
        for b in range(n_psi):
            if (y[a, b], x[a, b]) != (ref_y[a, b], ref_x[a, b]):
                m = raw[a, b]
                assert m[ref_y[a, b], ref_x[a, b]] >= m.max() - TIE_REL * abs(m.max())
