"""Search-text score modes against the reference's own scorer outputs
(golden_scorer.npz, written by tests/golden/make_golden_scorer.py)."""
from pathlib import Path

import numpy as np
import pytest

pytest.importorskip("scipy")

from gisapr_gb300 import scoring  # noqa: E402

GOLDEN = Path(__file__).resolve().parent / "golden" / "golden_scorer.npz"


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


def test_all_modes_match_reference(golden, tmp_path):
    texts = dict(zip([str(n) for n in golden["text_names"]], [str(t) for t in golden["texts"]]))
    for case, want in zip(golden["cases"], golden["outputs"]):
        name, cc, ss = str(case).split("|")
        path = tmp_path / f"{name}.txt"
        path.write_text(texts[name])
        got = scoring.run_this(str(path), float(cc), float(ss))
        np.testing.assert_allclose(np.asarray(got, dtype=np.float64), want, rtol=1e-9, atol=0, err_msg=str(case))


def test_simple_sum_equals_device_definition():
    """CC + simple sum is sum_i exp(rawCC_i / 1024), the score the engine reduces."""
    raw = np.asarray([300.0, 512.5, 100.25])
    lines = [str(["rawCC: ", 20 + i, float(r)]) + "\n" for i, r in enumerate(raw)]
    z, r = scoring.parse_search_values(lines)
    assert len(z) == 0 and np.array_equal(r, raw / 1024.0)
    assert scoring.score_values(z, r, 1, 1)[3] == pytest.approx(np.sum(np.exp(raw / 1024.0)), rel=1e-15)


def test_main_writes_index_results(golden, tmp_path):
    texts = dict(zip([str(n) for n in golden["text_names"]], [str(t) for t in golden["texts"]]))
    files = []
    for name in ("mixture", "empty"):
        p = tmp_path / f"{name}.txt"
        p.write_text(texts[name])
        files.append(str(p))
    index = tmp_path / "index.txt"
    index.write_text("\n".join(files) + "\n")
    out = tmp_path / "scores.txt"
    scoring.main([str(index), "1", "1", str(out)])
    lines = out.read_text().splitlines()
    assert lines[0] == files[0] and lines[2] == files[1] and lines[3] == "0.0 0.0 0.0"
    total, zval, ccval = (float(v) for v in lines[1].split())
    cases = [str(c) for c in golden["cases"]]
    want = golden["outputs"][cases.index("mixture|1.0|1.0")]
    assert total == pytest.approx(want[3], rel=1e-9) and zval == 0.0 and ccval == pytest.approx(want[1], rel=1e-9)
