"""The STAR readers against the reference's own (tests/golden/
golden_star.json, written by make_golden_star.py with v606's
read_particle_table and read_model_angles): loop and label rules, row line
indices, missing labels and loops without rows."""
import json
from pathlib import Path

import pytest

from gisapr_gb300.tables import read_model_angles, read_particle_table

GOLDEN = Path(__file__).resolve().parent / "golden" / "golden_star.json"


def test_star_readers_match_reference(tmp_path):
    fx = json.loads(GOLDEN.read_text())
    for case in fx["cases"]:
        path = tmp_path / f"{case['name']}.star"
        path.write_text(fx["texts"][case["name"]])
        if case["particles"] == "error":
            with pytest.raises(ValueError):
                read_particle_table(str(path))
        else:
            t = read_particle_table(str(path))
            want = case["particles"]
            assert t.has_ctf == want["has_ctf"] and t.loop.first_row == want["data_start"], case["name"]
            got = [[r.line_index, r.image_name, r.rot, r.tilt, r.psi, r.defocus_u, r.defocus_v, r.defocus_angle]
                   for r in t.records]
            assert got == want["rows"], case["name"]
        if case["angles"] == "error":
            with pytest.raises(ValueError):
                read_model_angles(str(path))
        else:
            a = read_model_angles(str(path))
            assert (a.rot, a.tilt, a.psi) == (case["angles"]["rot"], case["angles"]["tilt"], case["angles"]["psi"])
