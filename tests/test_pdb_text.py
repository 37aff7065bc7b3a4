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


def test_rotation_matrices_equal_the_per_pose_matrices():
    """The vectorized rotation of a batch of poses gives, element for
    element, the matrices of the per-pose call (the batch engine copies
    them to the device as the pose of every slot)."""
    import numpy as np
    from gisapr_gb300.pdb_text import rotation_matrices, rotation_matrix
    rng = np.random.default_rng(11)
    poses = np.concatenate([rng.uniform(-180, 180, (40, 3)), rng.uniform(-5, 5, (40, 3))], axis=1)
    poses[0, :3] = 0.0
    got = rotation_matrices(poses)
    for p, m in zip(poses, got):
        assert np.array_equal(m, rotation_matrix(p))
    assert rotation_matrices(np.zeros((0, 6))).shape == (0, 3, 3)
    import pytest
    with pytest.raises(ValueError):
        rotation_matrices(np.full((2, 6), np.nan))
