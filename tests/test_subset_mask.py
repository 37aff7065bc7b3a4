"""Host-side form of per-slot particle subsets (engine.subset_mask)."""
import numpy as np
import pytest

pytest.importorskip("torch")
from gisapr_gb300.engine import subset_mask  # noqa: E402


def test_forms():
    m = subset_mask([None, [3, 0], np.array([True, False, True, False, False]), []], 5, 5)
    assert m.dtype == np.uint8 and m.shape == (5, 5)
    np.testing.assert_array_equal(m[0], 1)
    np.testing.assert_array_equal(m[1], [1, 0, 0, 1, 0])
    np.testing.assert_array_equal(m[2], [1, 0, 1, 0, 0])
    np.testing.assert_array_equal(m[3], 0)
    np.testing.assert_array_equal(m[4], 1)   # slots past the list score every particle
    np.testing.assert_array_equal(subset_mask(None, 2, 3), 1)


@pytest.mark.parametrize("bad", [[[5]], [[-1]], [[1, 1]], [np.array([True, False])], [None] * 6])
def test_rejects(bad):
    with pytest.raises(ValueError):
        subset_mask(bad, 5, 5)
