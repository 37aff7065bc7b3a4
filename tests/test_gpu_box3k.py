"""Boxes 96 and 192 (3 * 2^k: a radix-3 pass over radix-2 shared-memory
transforms) on the GPU, through the C ABI, against the CPU oracle: templates,
particle spectra, the end-to-end score and the tensor-core forms. Box 256
templates (slice gather and row inverse in their own kernel, the remaining
passes in the general projector) against the oracle as well."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from gisapr_gb300 import synthetic as syn  # noqa: E402
from gisapr_gb300.engine import BatchScoringJob, JobConfig, ScoringJob  # noqa: E402
from gisapr_gb300.search import (IntegratedProjector, PackedFourierLayout, ParticleFourierPreparer,  # noqa: E402
                                 PsiGridBank)
from gisapr_gb300.tables import model_angles_from_lists  # noqa: E402
from oracle import gisapr_oracle as O  # noqa: E402
from tests.helpers import PEAK_REL, SCORE_REL, SPECTRUM_RRMS, TEMPLATE_RRMS, records_from_job, rrms  # noqa: E402

DEV = "cuda:0"


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__ as g
    g.build()


def _t(a):
    return torch.as_tensor(np.ascontiguousarray(a)).to(DEV)


@pytest.mark.parametrize("n,n_dir", [(96, 8), (192, 3), (256, 2)])
def test_templates_vs_oracle(n, n_dir):
    rng = np.random.default_rng(n)
    vol = syn.blob_density(n, n)  # blobs plus white noise: no shell near float32 rounding
    rot = rng.uniform(-180.0, 180.0, n_dir)
    tilt = np.rad2deg(np.arccos(rng.uniform(-1.0, 1.0, n_dir)))
    angles = model_angles_from_lists(rot, tilt)
    mask = O.soft_mask(n, int(round(0.43 * n)), 6)
    fsc = syn.logistic_fsc(n, 1.1, 4.0)
    packed_fsc = np.ascontiguousarray(O.centered_to_packed(O.radial_map(fsc, n)))
    proj = IntegratedProjector(DEV, n, n, PackedFourierLayout(n, 8, DEV), _t(mask), _t(packed_fsc))
    tm = proj.build_templates(_t(vol), angles).cpu().numpy()
    dft = O.volume_spectrum(vol)
    rot_t = O.rotation_matrices_t(rot, tilt)
    for k in range(n_dir):
        ref = O.template_from_slice(O.central_slice(dft, rot_t[k], n), n, n, mask, packed_fsc)
        assert rrms(tm[k], ref) < TEMPLATE_RRMS, (k, rrms(tm[k], ref))


def test_particle_spectra_box96_vs_oracle():
    spec = syn.WORKLOADS["box96_tiny"]
    job = syn.make_job(spec, seed=11, n_particles=4)
    n = spec.box
    recs = records_from_job(job)
    from gisapr_gb300.search import PackedCTFTorch
    ctf = PackedCTFTorch(n, spec.apix, spec.cs, spec.voltage, spec.kk, DEV).batch(recs, True)
    psis = [O.psi_sampling(r.psi, spec.psi_step, True, spec.local_range)[1] for r in recs]
    uniq = list(dict.fromkeys(float(np.round(a, 6)) for row in psis for a in row))
    bank = PsiGridBank(n, DEV, uniq)
    mask = O.soft_mask(n, spec.mask_radius, spec.mask_edge)
    prep = ParticleFourierPreparer(n, n, DEV, PackedFourierLayout(n, 8, DEV), _t(mask), bank)
    idx = torch.stack([bank.indices_for_angles(row) for row in psis])
    out = prep.prepare_batch(_t(job.images), idx, ctf).cpu().numpy()
    ctf_h = ctf.cpu().numpy()
    for i in range(len(recs)):
        ref = O.prepare_particle(job.images[i], psis[i], ctf_h[i], mask, n)
        assert rrms(out[i], ref) < SPECTRUM_RRMS, (i, rrms(out[i], ref))


def _box96_job():
    spec = syn.WORKLOADS["box96_tiny"]
    data = syn.make_job(spec, seed=21)
    cfg = JobConfig(box=spec.box, apix=spec.apix, crop=spec.crop, psi_step=spec.psi_step,
                    local_range=spec.local_range, mask_edge=spec.mask_edge, kk=spec.kk)
    job = ScoringJob(cfg, data.model.pdb_text, model_angles_from_lists(data.model_rot, data.model_tilt),
                     records_from_job(data), data.images, fsc_values=data.fsc, device=DEV)
    return spec, data, job


def test_scoring_job_box96_vs_oracle():
    spec, data, job = _box96_job()
    pose = syn.candidate_poses(1, 22, 3.0, 1.5, exact=True)[0]
    score = job.score(pose)
    rd = data.records
    ora = O.evaluate_candidate(data.model.pdb_text, pose, spec.box, spec.apix, spec.res, data.model_rot,
                               data.model_tilt, data.images, rd.line_index, rd.rot, rd.tilt, rd.psi, rd.defocus_u,
                               rd.defocus_v, rd.defocus_angle, data.fsc, spec.mask_radius, spec.mask_edge,
                               spec.psi_step, spec.local_range, spec.crop, kk=spec.kk, keep_templates=False)
    assert abs(score / ora["score"] - 1.0) < SCORE_REL
    r = job.particle_results()
    valid = r["best_entry"] >= 0
    np.testing.assert_allclose(r["peak"][valid], ora["raw"], rtol=PEAK_REL)
    assert job.score(pose) == score


@pytest.mark.parametrize("precision", ["fp16x3", "fp16"])
def test_tensor_core_forms_box96(precision):
    spec, data, job = _box96_job()
    poses = list(syn.candidate_poses(3, 23, 3.0, 1.5, exact=True))
    ref = BatchScoringJob(job, len(poses), use_graph=False, precision="fp32").score_active(poses)
    got = BatchScoringJob(job, len(poses), use_graph=False, precision=precision).score_active(poses)
    tol = 1e-5 if precision == "fp16x3" else 1e-4
    np.testing.assert_allclose(got, ref, rtol=tol)
    single = np.asarray([job.score(p) for p in poses])
    np.testing.assert_allclose(ref, single, rtol=1e-6)


@pytest.mark.parametrize("n", [32, 64, 128, 256])
def test_blocked_volume_transform_equals_cufft_path(n):
    """The blocked volume transform of power-of-two boxes (two N-point FFTs
    per 2N-point line of N nonzero samples, written in the gather's blocked
    layout) gives the templates of the cuFFT spectrum + blocked copy."""
    rng = np.random.default_rng(n + 1)
    vol = syn.blob_density(n, n + 3)
    n_dir = 6
    rot = rng.uniform(-180.0, 180.0, n_dir)
    tilt = np.rad2deg(np.arccos(rng.uniform(-1.0, 1.0, n_dir)))
    angles = model_angles_from_lists(rot, tilt)
    mask = O.soft_mask(n, int(round(0.43 * n)), 6)
    packed_fsc = np.ascontiguousarray(O.centered_to_packed(O.radial_map(syn.logistic_fsc(n, 1.1, 4.0), n)))
    proj = IntegratedProjector(DEV, n, n, PackedFourierLayout(n, 8, DEV), _t(mask), _t(packed_fsc))
    assert proj.blocked_fft
    fast = proj.build_templates(_t(vol), angles).cpu().numpy()
    proj.blocked_fft = False
    ref = proj.build_templates(_t(vol), angles).cpu().numpy()
    errs = [rrms(fast[k], ref[k]) for k in range(n_dir)]
    print(f"box {n}: blocked transform vs cuFFT path, max template rRMS {max(errs):.2e}")
    assert max(errs) < 3e-5, errs
