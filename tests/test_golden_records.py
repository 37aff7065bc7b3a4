"""Search-text records (the oracle's and the product's formatter) against the
reference's own make_result_records (v606:1452-1516) at crop 14 / scale 0.5,
crop 12 / scale 2/3 (half-integer shifts) and crop 10 / scale 1, with tied
maxima (tests/golden/make_golden_records.py; inputs regenerated from its
seeds)."""
import json
import sys
import types
from pathlib import Path

import numpy as np
import pytest

from gisapr_gb300 import synthetic as syn
from gisapr_gb300.search import format_records
from gisapr_gb300.tables import psi_sampling_for_record
from oracle import gisapr_oracle as O

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
from make_golden_records import CASES, HEALPIX_ORDER, case_inputs  # noqa: E402

GOLDEN = Path(__file__).resolve().parent / "golden" / "golden_records.json"


def _same(got, want):
    """Rows equal field by field; the z-score (float32 in the reference,
    float64 here) within 1e-5 relative, the angular distance within 1e-9."""
    assert [r[0] for r in got] == [r[0] for r in want]
    g0, w0 = got[0], want[0]
    assert g0[1] == w0[1] and g0[3:7] == w0[3:7] and g0[8:] == w0[8:]
    assert g0[2] == pytest.approx(w0[2], rel=1e-5, abs=1e-6)
    assert g0[7] == pytest.approx(w0[7], abs=1e-9)
    assert got[1] == want[1]
    assert got[2][:2] == want[2][:2] and got[2][2] == pytest.approx(want[2][2], rel=1e-7)


@pytest.mark.parametrize("k", range(len(CASES)))
def test_records_match_reference(k):
    golden = json.loads(GOLDEN.read_text())[k]
    crop, scale, step, local, n, seed = CASES[k]
    assert golden["case"] == [crop, scale, step, local, n, seed]
    m_rot, m_tilt = syn.healpix_directions(HEALPIX_ORDER)
    for (rec, dirs, scores, ys, xs), want in zip(case_inputs(crop, n, seed, len(m_rot)), golden["records"]):
        fake, _ = psi_sampling_for_record(rec["psi"], step, True, local)
        ora = O.result_record(rec["line_index"], rec["rot"], rec["tilt"], rec["psi"], fake, m_rot, m_tilt, dirs,
                              scores, ys, xs, crop, scale)
        _same(ora, want)
        flat = scores.reshape(-1)
        j = int(np.argmax(flat))                                  # first maximum, as the records kernel
        li, pi = divmod(j, scores.shape[1])
        f64 = flat.astype(np.float64)
        z = (f64[j] - f64.mean()) / f64.std()
        got = format_records(types.SimpleNamespace(**rec), fake, m_rot, m_tilt, dirs, li, pi, float(flat[j]),
                             int(ys[li, pi]), int(xs[li, pi]), z, crop, scale)
        _same(got, want)
