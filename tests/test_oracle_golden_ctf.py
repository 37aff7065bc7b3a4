"""The oracle's packed CTF * ISSPA table against both of the reference's
backends (PackedCTFTorch and PackedCTFNumPy, v606:695-829) at the boxes,
pixel sizes and ISSPA constants of the larger configurations
(tests/golden/make_golden_ctf.py; defocus values regenerated from its seeds)."""
import sys
from pathlib import Path

import numpy as np
import pytest

from oracle import gisapr_oracle as O
from tests.helpers import CTF_ABS

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
from make_golden_ctf import CASES, CS, VOLTAGE, case_defocus, rows  # noqa: E402

GOLDEN = Path(__file__).resolve().parent / "golden" / "golden_ctf.npz"


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


@pytest.mark.parametrize("k", range(len(CASES)))
def test_oracle_ctf_matches_both_reference_backends(golden, k):
    n, apix, kk, seed = CASES[k]
    assert tuple(golden[f"case{k}"]) == (n, apix, kk, seed)
    gen = O.PackedCTF(n, apix, CS, VOLTAGE, kk)
    ctf = np.stack([gen.one(u, v, a) for u, v, a in case_defocus(seed)])[:, rows(n)]
    # the numpy backend repeats the same float32 operations; torch's
    # vectorised sin/exp differ in the last bits (measured up to 1.3e-6)
    assert np.max(np.abs(ctf - golden[f"numpy{k}"])) < 1e-7
    assert np.max(np.abs(ctf - golden[f"torch{k}"])) < CTF_ABS
