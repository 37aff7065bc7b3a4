"""Batched candidates (one graph per batch) against the per-candidate path."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from gisapr_gb300 import synthetic as syn  # noqa: E402
from gisapr_gb300.engine import BatchScoringJob, JobConfig, ScoringJob  # noqa: E402
from gisapr_gb300.pdb2mrc import MovedChainDensity  # noqa: E402
from gisapr_gb300.tables import model_angles_from_lists  # noqa: E402
from tests.helpers import records_from_golden, records_from_job  # noqa: E402

DEV = "cuda:0"


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import __graft_entry__ as g
    g.build()


def _cfg(spec):
    return JobConfig(box=spec.box, apix=spec.apix, crop=spec.crop, psi_step=spec.psi_step,
                     local_range=spec.local_range, mask_edge=spec.mask_edge, kk=spec.kk)


@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_equals_single_candidates(golden32, use_graph):
    g = golden32
    spec = syn.WORKLOADS["box32_tiny"]
    job = ScoringJob(_cfg(spec), str(g["pdb_text"]), model_angles_from_lists(g["model_rot"], g["model_tilt"]),
                     records_from_golden(g), g["images"], fsc_values=g["fsc"], device=DEV)
    poses = [g["pose"]] + list(syn.candidate_poses(4, 3, 5.0, 3.0))
    single = np.asarray([job.score(p) for p in poses])
    single_peaks = []
    for p in poses:
        job.score(p)
        single_peaks.append(job.particle_results()["peak"])
    batch = BatchScoringJob(job, len(poses), use_graph=use_graph)
    got = batch.score_batch(poses)
    np.testing.assert_array_equal(got, single)
    np.testing.assert_array_equal(batch.peak.cpu().numpy(), np.stack(single_peaks))
    # a second generation through the same graph
    poses2 = list(syn.candidate_poses(5, 9, 5.0, 3.0))
    got2 = batch.score_batch(poses2)
    np.testing.assert_array_equal(got2, np.asarray([job.score(p) for p in poses2]))


def test_batch_mixes_moving_chains_of_different_sizes():
    spec = syn.WORKLOADS["box32_tiny"]
    models = syn.make_models_shared_fixed([120, 200, 320], 600, seed=4)
    data = syn.make_job(spec, seed=8, n_particles=10, model=models[1])
    angles = model_angles_from_lists(data.model_rot, data.model_tilt)
    recs = records_from_job(data)
    jobs = [ScoringJob(_cfg(spec), m.pdb_text, angles, recs, data.images, fsc_values=data.fsc, device=DEV)
            for m in models]
    dens = [MovedChainDensity(m.pdb_text, "A", spec.box, spec.apix, spec.res, DEV, from_text=True) for m in models]
    np.testing.assert_array_equal(dens[0].fixed.cpu().numpy(), dens[2].fixed.cpu().numpy())
    model_of = [0, 1, 2, 2, 1, 0]
    poses = list(syn.candidate_poses(len(model_of), 11, 5.0, 3.0))
    batch = BatchScoringJob(jobs[1], len(model_of), models=dens, model_of=model_of)
    got = batch.score_batch(poses)
    want = np.asarray([jobs[m].score(p) for m, p in zip(model_of, poses)])
    np.testing.assert_array_equal(got, want)


@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_lanes_equal_single_candidates_box96(use_graph):
    """Box 96 runs the cuFFT volume transform: the batch's two template
    lanes transform and project different candidates at the same time, each
    into its own context's spectrum, so every candidate's score and peaks
    equal the per-candidate path's bit for bit."""
    spec = syn.WORKLOADS["box96_tiny"]
    data = syn.make_job(spec, seed=5, n_particles=24)
    job = ScoringJob(_cfg(spec), data.model.pdb_text, model_angles_from_lists(data.model_rot, data.model_tilt),
                     records_from_job(data), data.images, fsc_values=data.fsc, device=DEV)
    poses = list(syn.candidate_poses(12, 21, 5.0, 3.0))
    single, single_peaks = [], []
    for p in poses:
        single.append(job.score(p))
        single_peaks.append(job.particle_results()["peak"])
    batch = BatchScoringJob(job, len(poses), use_graph=use_graph, lanes=2)
    for _ in range(2):
        got = batch.score_batch(poses)
        np.testing.assert_array_equal(got, np.asarray(single))
        np.testing.assert_array_equal(batch.peak.cpu().numpy(), np.stack(single_peaks))
