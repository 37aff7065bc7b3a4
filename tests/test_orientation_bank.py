"""Orientation banks are interchangeable with the reference's: the fixture
(tests/golden/golden_bank.json, written by make_golden_bank.py with the Lite
tree's own orientation_bank_v1) holds a bank the reference wrote; this
package must read it, compute the same settings, digest and rows, write the
same bank, and accept or reject the same restricted rows."""
import json
from pathlib import Path
from types import SimpleNamespace

import numpy as np
import pytest

from gisapr_gb300 import orientation_bank as ob
from gisapr_gb300.tables import read_model_angles, read_particle_table

GOLDEN = Path(__file__).resolve().parent / "golden" / "golden_bank.json"


@pytest.fixture(scope="module")
def fx():
    return json.loads(GOLDEN.read_text())


@pytest.fixture()
def files(tmp_path, fx):
    (tmp_path / "p.star").write_text(fx["particle_star"])
    (tmp_path / "a.star").write_text(fx["angle_star"])
    return tmp_path / "p.star", tmp_path / "a.star"


def test_settings_and_digest_match_reference(fx, files):
    p, a = files
    s = ob.bank_settings(p, a, fx["keep"], fx["local"], fx["local_range"], fx["psi_step"])
    assert s == fx["bank"]["settings"]
    assert ob.bank_digest(fx["bank"]) == fx["bank"]["sha256"]
    ob.check_bank(fx["bank"], s)


def test_rows_and_packed_bank_match_reference(fx, files):
    p, a = files
    angles = read_model_angles(str(a))
    table = read_particle_table(str(p))
    rows = {}
    for inp, rec in zip(fx["inputs"], table.records):
        assert rec.line_index == inp["line"] and rec.image_name == inp["image"]
        peaks = np.asarray(inp["scores"], np.float32).max(axis=1)
        rows[str(rec.line_index)] = ob.ranked_row(rec, inp["indices"], angles, peaks, fx["keep"])
    assert rows == fx["bank"]["rows"]
    s = ob.bank_settings(p, a, fx["keep"], fx["local"], fx["local_range"], fx["psi_step"])
    bank = ob.pack_bank(s, rows, mrc="/data/model.mrc")
    assert json.dumps(bank, sort_keys=True) == json.dumps(fx["bank"], sort_keys=True)


def test_read_write_and_tamper(fx, files, tmp_path):
    p, a = files
    s = ob.bank_settings(p, a, fx["keep"], fx["local"], fx["local_range"], fx["psi_step"])
    out = tmp_path / "sub" / "bank.json"
    ob.write_bank(out, fx["bank"])
    assert ob.read_bank(out, s) == fx["bank"]["rows"]
    assert [q.name for q in out.parent.iterdir()] == ["bank.json"]  # no temporary file left
    bad = json.loads(out.read_text())
    first = next(iter(bad["rows"]))
    bad["rows"][first]["directions"][0][3] += 1.0
    out.write_text(json.dumps(bad))
    with pytest.raises(ValueError, match="digest"):
        ob.read_bank(out, s)
    other = dict(s, keep=s["keep"] + 1)
    with pytest.raises(ValueError, match="settings"):
        ob.check_bank(fx["bank"], other)


def test_restricted_indices_match_reference(fx, files):
    _, a = files
    angles = read_model_angles(str(a))
    images = {inp["line"]: inp["image"] for inp in fx["inputs"]}
    for case in fx["restricted"]:
        rec = SimpleNamespace(line_index=case["line"], image_name=images[case["line"]])
        if case["result"] == "error":
            with pytest.raises(ValueError):
                ob.restricted_indices(case["row"], rec, case["allowed"], angles, fx["keep"])
        else:
            assert ob.restricted_indices(case["row"], rec, case["allowed"], angles, fx["keep"]) == case["result"]
