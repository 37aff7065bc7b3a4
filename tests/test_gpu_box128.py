"""The benchmarked configuration on the GPU, through the C ABI, against the
reference's own outputs (tests/golden/golden_box128.npz: box 128 at 1.1 A/px,
3,000 + 20,000 atoms, logistic FSC, HEALPix order 3 within +-10 degrees, psi
step 7.5, crop 12; 160 particles, 517 needed directions) and the FP64 oracle:
density, templates (the box-128 shared-memory projector), particle spectra,
every per-map maximum, per-particle (direction, psi, y, x) identical or tied
within 1e-5, peaks, z-scores and the candidate score, for the single
candidate path and the batched FP32 and tensor-core forms."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from gisapr_gb300.engine import BatchScoringJob, JobConfig, ScoringJob  # noqa: E402
from gisapr_gb300.pdb2mrc import MovedChainDensity  # noqa: E402
from gisapr_gb300.search import IntegratedProjector, PackedFourierLayout  # noqa: E402
from gisapr_gb300.tables import model_angles_from_lists  # noqa: E402
from oracle import gisapr_oracle as O  # noqa: E402
from tests.helpers import (DENSITY_RRMS, PEAK_REL, SCORE_REL, SPECTRUM_RRMS, TEMPLATE_RRMS_SMOOTH,  # noqa: E402
                           argmax_mismatches, oracle_window, records_from_job, rrms, template_ref_rrms)

DEV = "cuda:0"


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__ as g
    g.build()


@pytest.fixture(scope="module")
def job128(box128_case):
    spec, data, _ = box128_case
    cfg = JobConfig(box=spec.box, apix=spec.apix, crop=spec.crop, psi_step=spec.psi_step,
                    local_range=spec.local_range, mask_edge=spec.mask_edge, kk=spec.kk)
    return ScoringJob(cfg, data.model.pdb_text, model_angles_from_lists(data.model_rot, data.model_tilt),
                      records_from_job(data), data.images, fsc_values=data.fsc, device=DEV)


def _t(a):
    return torch.as_tensor(np.ascontiguousarray(a)).to(DEV)


def test_box128_density(golden128, box128_case):
    spec, data, ora = box128_case
    g = golden128
    dens = MovedChainDensity(data.model.pdb_text, "A", spec.box, spec.apix, spec.res, device=DEV, from_text=True)
    vol = dens.generate(g["pose"]).cpu().numpy()
    assert rrms(vol[62:66], g["density_slab"]) < DENSITY_RRMS
    assert rrms(vol, ora["density"]) < DENSITY_RRMS
    d = vol.astype(np.float64)
    np.testing.assert_allclose([d.sum(), (d ** 2).sum()], g["density_checksum"], rtol=1e-5)


def test_box128_templates(golden128, box128_case):
    """The shared-memory projector at box 128 (its own template instances)
    on the oracle's density: within 2.5e-4 relative RMS of the FP64 oracle
    (the float32 floor of this smooth density, see TEMPLATE_RRMS_SMOOTH) and
    within the reference's own float32 floor of the reference's templates."""
    spec, data, ora = box128_case
    g = golden128
    n = spec.box
    angles = model_angles_from_lists(data.model_rot, data.model_tilt)
    mask = O.soft_mask(n, spec.mask_radius, spec.mask_edge)
    packed_fsc = np.ascontiguousarray(O.centered_to_packed(O.radial_map(data.fsc, n)))
    proj = IntegratedProjector(DEV, n, n, PackedFourierLayout(n, spec.crop, DEV), _t(mask), _t(packed_fsc))
    sel = [int(k) for k in g["template_index"]]
    tm = proj.build_templates(_t(ora["density"].astype(np.float32)), angles, orientation_indices=sel).cpu().numpy()
    e_or = [rrms(tm[i], ora["templates"][k]) for i, k in enumerate(sel)]
    e_ref = [rrms(tm[i], g["templates"][i]) for i in range(len(sel))]
    print(f"box 128 templates: max rRMS {max(e_or):.2e} from the oracle, {max(e_ref):.2e} from the reference")
    assert max(e_or) < TEMPLATE_RRMS_SMOOTH, e_or
    assert max(e_ref) < template_ref_rrms(n), e_ref
    np.testing.assert_allclose(np.sqrt((np.abs(tm) ** 2).sum(axis=(1, 2))), 1.0, rtol=1e-5)


def test_box128_particle_spectra(golden128, box128_case, job128):
    _, _, ora = box128_case
    g = golden128
    stack = job128.stack
    for k, i in enumerate(g["particle_index"]):
        got = stack[int(i)].cpu().numpy()
        assert rrms(got, g["spectra"][k]) < SPECTRUM_RRMS
        assert rrms(got, ora["particles"][int(i)]["spectra"]) < SPECTRUM_RRMS


def _check_records(g, ora, spec, ptr, n_psi, r, scores=None):
    valid = r["best_entry"] >= 0
    np.testing.assert_allclose(r["peak"][valid], ora["raw"], rtol=PEAK_REL)
    np.testing.assert_allclose(r["peak"][valid], g["peak"], rtol=2 * PEAK_REL)
    np.testing.assert_allclose(r["zscore"][valid], g["z"], atol=2e-3)
    bad = argmax_mismatches(ptr, n_psi, g["scores"], g["ys"], g["xs"], r["best_entry"], r["best_psi"],
                            r["peak_y"], r["peak_x"], window=oracle_window(ora, spec.crop))
    assert not bad, bad
    if scores is not None:
        # every map maximum within 1e-4 of the particle's scale from the oracle
        oracle_maps = np.concatenate([p["scores"].reshape(-1) for p in ora["particles"] if len(p["local"])])
        for i in range(len(ptr) - 1):
            a, b = n_psi * ptr[i], n_psi * ptr[i + 1]
            if b > a:
                scale = np.max(np.abs(oracle_maps[a:b]))
                assert np.max(np.abs(scores[a:b] - oracle_maps[a:b])) <= PEAK_REL * scale, i


def test_box128_scoring_job(golden128, box128_case, job128):
    spec, _, ora = box128_case
    g = golden128
    job = job128
    ptr = job.local_ptr.cpu().numpy()
    np.testing.assert_array_equal(ptr, g["local_ptr"])
    np.testing.assert_array_equal(np.asarray(job.needed)[job.local_idx.cpu().numpy()], g["local_idx"])
    score = job.score(g["pose"])
    assert abs(score / float(g["score"]) - 1.0) < SCORE_REL
    assert abs(score / ora["score"] - 1.0) < SCORE_REL
    r = job.particle_results()
    _check_records(g, ora, spec, ptr, job.n_psi, r, scores=job.score_buf.cpu().numpy())
    assert job.score(g["pose"]) == score


@pytest.mark.parametrize("precision", ["fp32", "fp16x3"])
def test_box128_batched_forms(golden128, box128_case, job128, precision):
    """A batch of two slots (the fixture's pose and a second pose): the
    fixture's slot gives the reference's records in the FP32 and split
    tensor-core forms alike."""
    spec, _, ora = box128_case
    g = golden128
    job = job128
    from gisapr_gb300 import synthetic as syn
    poses = [g["pose"], syn.candidate_poses(1, 77, 3.0, 1.5, exact=True)[0]]
    b = BatchScoringJob(job, 2, use_graph=False, precision=precision)
    scores = b.score_active(poses)
    assert abs(scores[0] / float(g["score"]) - 1.0) < SCORE_REL
    assert abs(scores[0] / ora["score"] - 1.0) < SCORE_REL
    single = job.score(poses[1])
    assert abs(scores[1] / single - 1.0) < (1e-6 if precision == "fp32" else 1e-5)
    r = b.slot_results(1)[0]
    _check_records(g, ora, spec, job.local_ptr.cpu().numpy(), job.n_psi, r,
                   scores=b.score_buf[0].cpu().numpy())
