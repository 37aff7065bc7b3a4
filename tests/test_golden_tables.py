"""Local direction lists and psi sampling (the product's host tables and the
oracle) against the reference's own build_local_orientation_entries and
psi_sampling_for_record (v606:331-378, 1163-1190) at HEALPix order 3 within
+-10 degrees / psi 7.5 and order 4 within +-6 degrees / psi 3.75
(tests/golden/make_golden_tables.py; particle angles regenerated from its
seeds)."""
import sys
import types
from pathlib import Path

import numpy as np
import pytest

from gisapr_gb300 import synthetic as syn
from gisapr_gb300.tables import build_local_orientation_entries, psi_sampling_for_record
from oracle import gisapr_oracle as O

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
from make_golden_tables import CASES, case_particles  # noqa: E402

GOLDEN = Path(__file__).resolve().parent / "golden" / "golden_tables.npz"


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


@pytest.mark.parametrize("k", range(len(CASES)))
def test_local_lists_and_psi_match_reference(golden, k):
    order, local, step, n, seed = CASES[k]
    m_rot, m_tilt = syn.healpix_directions(order)
    rot, tilt, psi = case_particles(n, seed)
    ptr, idx = golden[f"ptr{k}"], golden[f"idx{k}"]
    want = [idx[ptr[i]:ptr[i + 1]].tolist() for i in range(n)]
    recs = [types.SimpleNamespace(line_index=i + 10, rot=float(r), tilt=float(t), psi=float(p))
            for i, (r, t, p) in enumerate(zip(rot, tilt, psi))]
    got = build_local_orientation_entries(recs, m_rot, m_tilt, local)
    assert [e[0] for e in got] == [i + 10 for i in range(n)]
    assert [list(e[1:]) for e in got] == want
    assert O.local_orientations(rot, tilt, m_rot, m_tilt, local) == want
    for i in range(n):
        fake, eff = psi_sampling_for_record(float(psi[i]), step, True, local)
        np.testing.assert_array_equal(fake, golden[f"fake{k}"][i])
        np.testing.assert_array_equal(eff, golden[f"eff{k}"][i])
        of, oe = O.psi_sampling(float(psi[i]), step, True, local)
        np.testing.assert_array_equal(of, golden[f"fake{k}"][i])
        np.testing.assert_array_equal(oe, golden[f"eff{k}"][i])
