"""The PDB reader against the reference's own reader (tests/golden/
golden_pdb.json, written by make_golden_pdb.py with GisAPR's pdb_text):
model spans, HETATM switch, element rules, chains, line indices, errors."""
import json
from pathlib import Path

import numpy as np
import pytest

from gisapr_gb300.pdb_text import read_pdb, read_pdb_text

GOLDEN = Path(__file__).resolve().parent / "golden" / "golden_pdb.json"


@pytest.fixture(scope="module")
def fx():
    return json.loads(GOLDEN.read_text())


def test_reader_matches_reference(fx, tmp_path):
    for case in fx["cases"]:
        text = fx["texts"][case["text"]]
        path = tmp_path / f"{case['text']}.pdb"
        path.write_text(text)
        kw = dict(include_hetatm=case["include_hetatm"], first_model_only=case["first_model_only"])
        if case["result"] == "error":
            with pytest.raises(ValueError):
                read_pdb(str(path), **kw)
            with pytest.raises(ValueError):
                read_pdb_text(text, **kw)
            continue
        for p in (read_pdb(str(path), **kw), read_pdb_text(text, **kw)):
            want = case["result"]
            assert p.coords.dtype == np.float32
            np.testing.assert_array_equal(p.coords.astype(float).reshape(-1, 3), np.asarray(want["coords"]).reshape(-1, 3))
            assert p.elements.tolist() == want["elements"], case
            assert p.chains.tolist() == want["chains"], case
            assert p.atom_line_indices.tolist() == want["lines"], case
