"""Pin the CPU oracle to the reference's own outputs (tests/golden/*.npz,
made by tests/golden/make_golden.py from GisAPR's code)."""
import numpy as np
import pytest

from gisapr_gb300 import synthetic as syn
from oracle import gisapr_oracle as O
from tests.helpers import (DENSITY_RRMS, PEAK_REL, SCORE_REL, SPECTRUM_RRMS, rrms)


@pytest.fixture(scope="module")
def box32_oracle(golden32):
    g = golden32
    spec = syn.WORKLOADS["box32_tiny"]
    return O.evaluate_candidate(str(g["pdb_text"]), g["pose"], spec.box, spec.apix, spec.res,
                                list(g["model_rot"]), list(g["model_tilt"]), g["images"], g["rec_line"],
                                g["rec_rot"], g["rec_tilt"], g["rec_psi"], g["rec_dfu"], g["rec_dfv"],
                                g["rec_dfa"], g["fsc"], spec.mask_radius, spec.mask_edge, spec.psi_step,
                                spec.local_range, spec.crop, kk=spec.kk)


def test_moved_coordinates_match_reference(golden32):
    g = golden32
    coords, z, chains = O.moved_density_atoms(str(g["pdb_text"]), "A", g["pose"])
    np.testing.assert_array_equal(coords, g["density_coords"])


def test_density(golden32, box32_oracle):
    assert rrms(box32_oracle["density"], golden32["density"]) < DENSITY_RRMS


def test_fixed_density(golden32):
    g = golden32
    c, e, ch = O.read_pdb_text(str(g["pdb_text"]))
    sel = ch != "A"
    d = O.splat_density(c[sel], O.atomic_numbers(e[sel]), 32, 3.0, 6.0)
    assert rrms(d, g["fixed_density"]) < DENSITY_RRMS


def test_rotation_matrices(golden32):
    np.testing.assert_array_equal(O.rotation_matrices_t(golden32["model_rot"], golden32["model_tilt"]),
                                  golden32["rot_t"])


def test_mask_and_fsc(golden32):
    np.testing.assert_array_equal(O.soft_mask(32, syn.WORKLOADS["box32_tiny"].mask_radius, 3), golden32["mask"])
    np.testing.assert_array_equal(O.centered_to_packed(O.radial_map(golden32["fsc"], 32)), golden32["packed_fsc"])


def test_ctf_matches_both_reference_backends(golden32):
    g = golden32
    gen = O.PackedCTF(32, 3.0, 2.7, 300.0, 3.0)
    ctf = np.stack([gen.one(u, v, a) for u, v, a in zip(g["rec_dfu"], g["rec_dfv"], g["rec_dfa"])])
    # the reference's numpy backend is the exact-layout reference (v606:549-692)
    assert np.max(np.abs(ctf - g["ctf_numpy"])) < 2e-6
    assert np.max(np.abs(ctf - g["ctf"])) < 2e-6


def test_local_lists_and_psi(golden32, box32_oracle):
    g = golden32
    ptr, idx = g["local_ptr"], g["local_idx"]
    ref_local = [list(idx[ptr[i]:ptr[i + 1]]) for i in range(len(ptr) - 1)]
    assert box32_oracle["local"] == ref_local
    for i, psi in enumerate(g["rec_psi"]):
        fake, eff = O.psi_sampling(float(psi), 15.0, True, 30.0)
        np.testing.assert_array_equal(fake, g["fake_psi"][i])
        np.testing.assert_array_equal(eff, g["eff_psi"][i])


def test_templates(golden32, box32_oracle):
    """The reference's float32 templates sit within 1e-4 relative RMS of the
    FP64 oracle; the residual is the reference's own float32 whitening error
    (weak high-frequency shells are rescaled to unit amplitude)."""
    errs = [rrms(t, golden32["templates"][k]) for k, t in box32_oracle["templates"].items()]
    assert max(errs) < 1e-4
    assert np.median(errs) < 4e-5


def test_particle_spectra(golden32, box32_oracle):
    for p, s in zip(box32_oracle["particles"], golden32["spectra"]):
        assert rrms(p["spectra"], s) < SPECTRUM_RRMS


def test_correlation_closed_form_matches_reference(golden32):
    """The crop-window closed form reproduces the reference's torch irfft2
    path on the reference's own templates and spectra."""
    g = golden32
    ptr, idx = g["local_ptr"], g["local_idx"]
    off = 0
    for i in range(len(ptr) - 1):
        loc = idx[ptr[i]:ptr[i + 1]]
        if len(loc) == 0:
            continue
        s, y, x = O.correlate(g["templates"][loc], g["spectra"][i], 8)
        n = s.size
        ref = g["scores"][off:off + n].reshape(s.shape)
        np.testing.assert_allclose(s, ref, rtol=2e-5, atol=1e-3)
        np.testing.assert_array_equal(y, g["ys"][off:off + n].reshape(s.shape))
        np.testing.assert_array_equal(x, g["xs"][off:off + n].reshape(s.shape))
        off += n


def test_records_and_score(golden32, box32_oracle):
    g = golden32
    raw = box32_oracle["raw"]
    assert np.max(np.abs(raw / g["peak"] - 1.0)) < PEAK_REL
    assert abs(box32_oracle["score"] / float(g["score"]) - 1.0) < SCORE_REL
    k = 0
    for p in box32_oracle["particles"]:
        if not p["local"]:
            continue
        cc, psi, rawr = p["records"]
        assert cc[5] == pytest.approx(float(g["best_dir"][k]) * 0 + cc[5])
        assert p["local"][int(np.argmax(p["scores"].reshape(-1))) // p["scores"].shape[1]] == g["best_dir"][k]
        assert cc[8] == g["shift_x"][k] and cc[9] == g["shift_y"][k]
        assert abs(cc[2] - g["z"][k]) < 1e-3 * max(1.0, abs(g["z"][k]))
        assert psi[2] == g["best_psi"][k]
        k += 1


def test_box64_published_cpu_configuration(golden64):
    """The CPU-sized published configuration: box 64 / 1.5 A, 200 particles,
    HEALPix order 2, +-15 deg, psi 15 deg, +-4 px."""
    g = golden64
    spec = syn.WORKLOADS["box64_200p"]
    job = syn.make_job(spec, seed=int(g["seed"]))
    chk = np.asarray([job.images.astype(np.float64).sum(), (job.images.astype(np.float64) ** 2).sum()])
    np.testing.assert_allclose(chk, g["image_checksum"], rtol=1e-6, atol=1e-3)
    r = job.records
    res = O.evaluate_candidate(job.model.pdb_text, g["pose"], spec.box, spec.apix, spec.res, job.model_rot,
                               job.model_tilt, job.images, r.line_index, r.rot, r.tilt, r.psi, r.defocus_u,
                               r.defocus_v, r.defocus_angle, job.fsc, spec.mask_radius, spec.mask_edge,
                               spec.psi_step, spec.local_range, spec.crop, kk=spec.kk)
    assert rrms(res["density"][28:36], g["density_slab"]) < DENSITY_RRMS
    for k, t in zip(g["template_index"], g["templates"]):
        if int(k) in res["templates"]:
            assert rrms(res["templates"][int(k)], t) < 2e-4
    for k, s in zip(g["particle_index"], g["spectra"]):
        assert rrms(res["particles"][int(k)]["spectra"], s) < SPECTRUM_RRMS
    assert np.max(np.abs(res["raw"] / g["peak"] - 1.0)) < PEAK_REL
    assert abs(res["score"] / float(g["score"]) - 1.0) < SCORE_REL
