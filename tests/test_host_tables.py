"""Host-side tables of the package against the oracle and the fixtures."""
import math

import numpy as np
import pytest

from gisapr_gb300 import synthetic as syn
from gisapr_gb300 import tables as T
from gisapr_gb300.pdb_text import quantize_coordinates, read_pdb_text, split_moving_chain, transform_coordinates
from oracle import gisapr_oracle as O
from tests.helpers import records_from_golden


def test_healpix_directions_match_fixture(golden32):
    rot, tilt = syn.healpix_directions(1)
    np.testing.assert_array_equal(rot, golden32["model_rot"])
    np.testing.assert_array_equal(tilt, golden32["model_tilt"])


def test_model_angles(golden32):
    a = T.model_angles_from_lists(golden32["model_rot"], golden32["model_tilt"])
    np.testing.assert_array_equal(a.rotation_matrices_t, golden32["rot_t"])


def test_local_orientation_entries(golden32):
    g = golden32
    recs = records_from_golden(g)
    ent = T.build_local_orientation_entries(recs, list(g["model_rot"]), list(g["model_tilt"]), 30.0)
    ptr, idx = g["local_ptr"], g["local_idx"]
    for i, e in enumerate(ent):
        assert e[0] == recs[i].line_index
        assert e[1:] == list(idx[ptr[i]:ptr[i + 1]])


def test_psi_sampling_and_table(golden32):
    g = golden32
    for i, psi in enumerate(g["rec_psi"]):
        fake, eff = T.psi_sampling_for_record(float(psi), 15.0, True, 30.0)
        assert fake == list(g["fake_psi"][i]) and eff == list(g["eff_psi"][i])
        assert (fake, eff) == O.psi_sampling(float(psi), 15.0, True, 30.0)
    # the rotation table rows reproduce the oracle's float32 grid coordinates
    for angle in (0.5, 7.5, 352.5, 123.0):
        c, s, o0, o1 = T.psi_rotation_entry(64, angle)
        py, px = O.psi_grid_pixels(64, angle)
        yy, xx = np.meshgrid(np.arange(64, dtype=np.float32), np.arange(64, dtype=np.float32), indexing="ij")
        sy = O._fma32(-s, xx, c * yy) + o0
        yn = np.float32(2.0) * sy / np.float32(63) - np.float32(1.0)
        np.testing.assert_array_equal((yn + np.float32(1)) * (np.float32(63) / np.float32(2)), py)


def test_mask_fsc_layout(golden32):
    np.testing.assert_array_equal(T.generate_soft_mask((32, 32), syn.WORKLOADS["box32_tiny"].mask_radius, 3),
                                  golden32["mask"])
    np.testing.assert_array_equal(T.centered_to_packed_np(T.expand_radial_values(golden32["fsc"], 32)),
                                  golden32["packed_fsc"])


def test_ctf_static_terms_match_oracle():
    st = T.ctf_static_terms(64, 1.5, 2.7, 300.0, 3.0)
    o = O.PackedCTF(64, 1.5, 2.7, 300.0, 3.0)
    for a, b in ((st.x, o.x), (st.y, o.y), (st.u4, o.u4), (st.ncurve, o.ncurve)):
        np.testing.assert_array_equal(a, b)
    assert (st.k1, st.k2, st.k3) == (float(o.k1), float(o.k2), float(o.k3))


def test_angular_distance_matches_oracle():
    rng = np.random.default_rng(0)
    for _ in range(50):
        a = rng.uniform(-180, 180, 6)
        assert T.calculate_angular_distance(*a) == O.angular_distance(*a)


def test_pdb_parse_and_pivot(golden32):
    text = str(golden32["pdb_text"])
    first = read_pdb_text(text)
    c, e, ch = O.read_pdb_text(text)
    np.testing.assert_array_equal(first.coords, c)
    split = split_moving_chain(first, "A", False, read_pdb_text(text, include_hetatm=False,
                                                                 first_model_only=False))
    assert split.pivot.dtype == np.float32
    np.testing.assert_array_equal(split.pivot, np.mean(c[ch == "A"], axis=0))


def test_quantize_matches_formatter():
    rng = np.random.default_rng(1)
    v = rng.uniform(-300, 300, (2000, 3))
    v[:20] = np.round(v[:20] * 1000) / 1000 + 0.0005  # near-ties
    np.testing.assert_array_equal(quantize_coordinates(v), O.quantize_8_3(v))


def test_moved_chain_matches_reference(golden32):
    text = str(golden32["pdb_text"])
    first = read_pdb_text(text)
    moved = transform_coordinates(first.coords[first.chains == "A"], golden32["pose"])
    np.testing.assert_allclose(moved, golden32["moved_float"], rtol=0, atol=1e-12)
