"""The FP64 reference of the bench's precision block (torch float64, run on
the CPU here) equals the oracle's closed form of the reference's
crop-window irfft2 on the same templates and particle spectra."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import bench  # noqa: E402
from oracle import gisapr_oracle as O  # noqa: E402


def test_fp64_maxima_match_the_oracle():
    rng = np.random.default_rng(5)
    n, crop, n_psi = 32, 6, 3
    h = n // 2 + 1
    bank = (rng.normal(size=(7, n, h)) + 1j * rng.normal(size=(7, n, h))).astype(np.complex64)
    stack = (rng.normal(size=(4, n_psi, n, h)) + 1j * rng.normal(size=(4, n_psi, n, h))).astype(np.complex64)
    ptr = np.array([0, 3, 3, 5, 8], np.int32)
    idx = np.array([0, 4, 6, 1, 2, 3, 5, 0], np.int32)
    got = bench.fp64_maxima(torch.from_numpy(bank), torch.from_numpy(stack), ptr, idx, 4, crop)
    assert got[1] is None
    for i in (0, 2, 3):
        s, y, x = O.correlate(bank[idx[ptr[i]:ptr[i + 1]]], stack[i], crop)
        np.testing.assert_allclose(got[i][0], s, rtol=1e-12, atol=1e-9)
        np.testing.assert_array_equal(got[i][1], y)
        np.testing.assert_array_equal(got[i][2], x)
